"""Generate the golden fixtures in tests/golden/ from the reference's own files.

Run once, in a container where the reference checkout exists, with the path
of that checkout (the ParallelTemperingMonteCarlo.jl package root):

    python tests/golden/make_golden.py <reference package root>

Outputs (committed, small):
  multihist_nvt.json  — the NVT Output literal and expected Cv values embedded in
                        test/multihist_test.jl:4-16 (R=32, 100 bins, thr 1e-3)
  multihist_npt.json  — the NPT Output literal and expected Cp values,
                        test/multihist_test.jl:18-32 (R=3, p=3.4439647528956955e-9)
  checkpoint_ne13.json — the Ne13 checkpoint fixture test/testing_data/checkpoint/
                        (params, hist_info, 25x102 histograms, 25 configurations)
  lookup_table_2.json — header, c6coeff and four entries of
                        scripts/lookup-tables/look-up_table-2.txt as read by
                        read_lookuptable (checked against test/test_potentials.jl:58-64)
  nn_cu55.json        — the symmetry-function table of scripts/cu55.jl:55-135
                        with the min/max scaling values of scripts/data/scaling.data
                        (rows 1:88, columns 3 = min and 4 = max), and the Cu55
                        icosahedral start geometry of scripts/cu55.jl:164-222
The reference itself is never read at test time; only these JSON files are.
"""
import json
import os
import re
import sys


def _tokenize(s):
    tok = re.compile(r"\s*(Matrix\{Float64\}\[\]|Vector\{Float64\}\[\]|Float64\[\]|"
                     r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?|\[|\]|,|;|\)|\n)")
    pos = 0
    out = []
    while pos < len(s):
        m = tok.match(s, pos)
        if not m:
            raise ValueError("cannot parse at %r" % s[pos:pos + 40])
        t = m.group(1)
        pos = m.end()
        out.append(t)
        if t == ")":
            break
    return out


def _parse_list(toks, i):
    """Parse a Julia array literal starting at toks[i] == '['.

    Returns (value, next index).  A vector gives a list; a matrix literal
    (rows separated by ';', elements by blanks) gives a list of rows."""
    assert toks[i] == "["
    i += 1
    items, rows, row = [], [], []
    is_matrix = False
    while True:
        t = toks[i]
        if t == "]":
            i += 1
            break
        if t == "[":
            v, i = _parse_list(toks, i)
            items.append(v)
            continue
        if t == ",":
            i += 1
            continue
        if t == ";":
            is_matrix = True
            rows.append(row)
            row = []
            i += 1
            continue
        if t == "\n":
            i += 1
            continue
        row.append(float(t))
        i += 1
    if is_matrix or (row and items == [] and False):
        rows.append(row)
        return rows, i
    if items:
        return items, i
    return row, i


def parse_output_literal(text, start):
    """Parse `Output{Float64}(a1, ..., a15)` beginning at text[start] == '('."""
    toks = _tokenize(text[start + 1:])
    args, i = [], 0
    while i < len(toks):
        t = toks[i]
        if t == ")":
            break
        if t in (",", "\n"):
            i += 1
            continue
        if t in ("Float64[]", "Matrix{Float64}[]", "Vector{Float64}[]"):
            args.append([])
            i += 1
            continue
        if t == "[":
            v, i = _parse_list(toks, i)
            args.append(v)
            continue
        args.append(float(t))
        i += 1
    return args


# The literal in test/multihist_test.jl predates lh_histogram: 15 arguments.
NAMES = ["n_bin", "en_min", "en_max", "v_min", "v_max", "max_displ", "en_avg",
         "heat_cap", "en_histogram", "ev_histogram", "rdf",
         "count_stat_atom", "count_stat_vol", "count_stat_rot", "count_stat_exc"]


def multihist(ref):
    text = open(os.path.join(ref, "test", "multihist_test.jl")).read()
    starts = [m.end() - 1 for m in re.finditer(r"Output\{Float64\}\(", text)]
    assert len(starts) == 2
    out = []
    for k, st in enumerate(starts):
        args = parse_output_literal(text, st)
        assert len(args) == 15, len(args)
        d = dict(zip(NAMES, args))
        seg = text[st: starts[1] if k == 0 else len(text)]
        exp = {int(a): float(b) for a, b in
               re.findall(r"@test c[vp]_?3?\[(\d+)\]\s*==\s*([-+0-9.eE]+)", seg)}
        d["expected"] = exp
        out.append(d)
    nvt, npt = out
    nvt.update({"R": 32, "t_i": 5.0, "t_f": 16.0, "thr": 1e-3, "n_atoms": 13})
    npt.update({"R": 3, "t_i": 20.0, "t_f": 40.0, "thr": 1e-3, "n_atoms": 32,
                "pressure": 3.4439647528956955e-9})
    # ev_histogram: list of R matrices, each (n_bin+2) rows
    return nvt, npt


def checkpoint(ref):
    d = os.path.join(ref, "test", "testing_data", "checkpoint")
    lines = open(os.path.join(d, "params.data")).read().split("\n")
    params = [float(x) for x in lines[1].split()]
    hist_info = [float(x) for x in open(os.path.join(d, "hist_info.data")).read().split("\n")[1].split()]
    hists = [[float(x) for x in ln.split()] for ln in
             open(os.path.join(d, "histograms.data")).read().strip().split("\n")]
    configs = []
    for i in range(1, 26):
        ls = open(os.path.join(d, "config.%d" % i)).read().strip().split("\n")
        n = int(ls[0])
        hdr = ls[1].split()
        xyz = [[float(v) for v in ln.split()[1:4]] for ln in ls[2:2 + n]]
        configs.append({"header": hdr, "xyz": xyz})
    index = int(open(os.path.join(d, "index.txt")).read().split()[0])
    pot = lines[4].split()
    return {"params": params, "ensemble": lines[3].split(), "potential": pot,
            "hist_info": hist_info, "histograms": hists, "configs": configs,
            "index": index}


def nn_tables(ref):
    src = open(os.path.join(ref, "scripts", "cu55.jl")).read()
    xm = re.search(r"X = \[(.*?)\]\n", src, re.S).group(1)
    X = [[float(v) for v in ln.split()] for ln in xm.strip().split("\n")]
    vm = re.search(r"V = \[(.*?)\n\]\n", src, re.S).group(1)
    V = [[float(v) for v in row.split(",")] for row in re.findall(r"\[([^\[\]]+)\]", vm)]
    T = [int(v) for v in re.search(r"T = \[([^\]]*)\]", src).group(1).split(",")]
    sc = [ln.split() for ln in open(os.path.join(ref, "scripts", "data", "scaling.data")).read().strip().split("\n")]
    gvals = [(float(r[2]), float(r[3])) for r in sc[:88]]   # (min, max)
    sf = []
    for k, row in enumerate(X):   # RadialType2(eta=row[2], r_cut=row[4], type=row[1])
        sf.append({"kind": 0, "type": int(row[0]), "eta": row[1], "lambda": 0.0, "zeta": 0.0,
                   "rcut": row[3], "gmin": gvals[k][0], "gmax": gvals[k][1]})
    n = len(X)
    for el in V:
        for ty in T:
            sf.append({"kind": 1, "type": ty, "eta": el[0], "lambda": el[1], "zeta": el[2],
                       "rcut": el[3], "gmin": gvals[n][0], "gmax": gvals[n][1]})
            n += 1
    ico = re.search(r"ico_55 = \[(.*?)\n\]\n", src, re.S).group(1)
    pos = [[float(v) for v in row.split(",")] for row in re.findall(r"\[([^\[\]]+)\]", ico)]
    assert len(sf) == 88 and len(pos) == 55
    return {"sf": sf, "ico55_nm": pos, "nm_to_bohr": 18.8973, "cu_lattice_nm": 0.36258}


def lookup_table(ref):
    """scripts/lookup-tables/look-up_table-2.txt read by the package's
    read_lookuptable (restating src/EnergyEvaluation.jl:227-256), checked
    against the known answers of test/test_potentials.jl:58-64; the header,
    c6coeff and a few table entries are kept (not the table)."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    import __graft_entry__ as g
    pk = g.load_package()
    path = os.path.join(ref, "scripts", "lookup-tables", "look-up_table-2.txt")
    table, sd, sa, ld, la, dd, da, c6 = pk.read_lookuptable(path)
    assert table[0, 0] == 282.19449125205114 and sd == 0.1 and sa == 0
    assert table.size == la * ld
    samples = [[i, j, float(table[i, j])] for i, j in ((0, 0), (0, 999), (45, 500), (90, ld - 1))]
    return {"file": "scripts/lookup-tables/look-up_table-2.txt", "l_dist": ld, "start_dist": sd,
            "d_dist": dd, "l_angle": la, "start_angle": sa, "d_angle": da, "c6coeff": c6,
            "samples": samples}


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <reference package root>")
    ref = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    nvt, npt = multihist(ref)
    json.dump(nvt, open(os.path.join(here, "multihist_nvt.json"), "w"))
    json.dump(npt, open(os.path.join(here, "multihist_npt.json"), "w"))
    json.dump(checkpoint(ref), open(os.path.join(here, "checkpoint_ne13.json"), "w"))
    json.dump(nn_tables(ref), open(os.path.join(here, "nn_cu55.json"), "w"), indent=0)
    json.dump(lookup_table(ref), open(os.path.join(here, "lookup_table_2.json"), "w"), indent=0)
    print("golden fixtures written to", here)


if __name__ == "__main__":
    main()
