"""A synthetic LookupTablePotential file in the reference's format
(src/EnergyEvaluation.jl:227-256): column j of angle row i holds the
ELJPotentialB dimer energy at r = start_dist + j d_dist and theta = (i - 1)
degrees, the values the table lookup is meant to return there."""
import math

import numpy as np

ELJB_A = [0.0005742, -0.4032, -0.2101, -0.0595, 0.0606, 0.1608]   # test/setup_params.jl:73-77
ELJB_B = [-0.01336, -0.02005, -0.1051, -0.1268, -0.1405, -0.1751]
ELJB_C = [-0.1132, -1.5012, 35.6955, -268.7494, 729.7605, -583.4203]


def eljb(r2, tn, a=ELJB_A, b=ELJB_B, c=ELJB_C):
    """dimer_energy of ELJPotentialB (src/EnergyEvaluation.jl:943-958)."""
    if not r2 >= 5.30:
        return 0.1
    r6inv = 1 / (r2 * r2 * r2)
    t2 = 2 / (tn * tn + 1) - 1
    t4 = 2 * (t2 * t2) - 1
    s = c[0] * r6inv * (1 + a[0] * t2 + b[0] * t4)
    r6inv /= r2
    for i in range(1, len(c)):
        s += c[i] * r6inv * (1 + a[i] * t2 + b[i] * t4)
        r6inv /= math.sqrt(r2)
    return s


def write_lut(path, l_dist=1491, start=0.1, dd=0.01, l_angle=91, da=1.0):
    with open(path, "w") as f:
        f.write("%d, %r, %r ! distances: count, first, step\n" % (l_dist, start, dd))
        f.write("%d, %r, %r ! angles\n" % (l_angle, 0.0, da))
        for i in range(l_angle):
            th = math.radians(i * da)
            tn = math.tan(th) if i * da < 90 else 1e300
            for j in range(1, l_dist + 1):
                r = start + j * dd
                f.write("%r\n" % eljb(r * r, tn))
    return path


def lut_energy_np(table, start, dd, da, c6, r2, tn):
    """The lookup of src/EnergyEvaluation.jl:277-298 restated in numpy."""
    la, ld = table.shape
    at = abs(tn)
    ia = 1
    if 0.00872687153 < at <= 114.592845357:
        ia = int(np.rint(math.atan(at) / da * 180.0 / math.pi + 1.0))
    elif at > 114.592845357:
        ia = 91
    ia = min(max(ia, 1), la)
    if r2 <= (start + 0.5 * dd) ** 2:
        return table[ia - 1, 0]
    if r2 <= (start + ld * dd) ** 2:
        jd = int(np.rint((math.sqrt(r2) - start) / dd))
        return table[ia - 1, min(max(jd, 1), ld) - 1]
    return c6 / (r2 * r2 * r2)
