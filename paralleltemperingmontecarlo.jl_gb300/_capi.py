"""ctypes binding of libptmc_gb300.so (include/ptmc_gb300.h).

The library is built in-tree by build.py.  Loading fails loudly when it is
missing or when no CUDA device is usable: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libptmc_gb300.so")

PTMC_OK = 0
ERRORS = {-1: "argument", -2: "state", -3: "cuda", -4: "sphere", -5: "io", -6: "limit"}
NVT, NPT, NNVT = 0, 1, 2
BC_SPHERE, BC_CUBIC, BC_RECTANGULAR, BC_RHOMBIC = 0, 1, 2, 3
FP64, FP32_RESYNC = 0, 1
TGEOMETRIC, TLINEAR = 0, 1

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)


class Params(ctypes.Structure):
    _fields_ = [("n_runs", ctypes.c_int), ("n_traj", ctypes.c_int),
                ("mc_cycles", ctypes.c_longlong), ("eq_cycles", ctypes.c_longlong),
                ("mc_sample", ctypes.c_int), ("n_adjust", ctypes.c_int), ("n_bin", ctypes.c_int),
                ("min_acc", ctypes.c_double), ("max_acc", ctypes.c_double),
                ("ensemble", ctypes.c_int), ("pressure", ctypes.c_double),
                ("t_i", ctypes.c_double), ("t_f", ctypes.c_double), ("tdistr", ctypes.c_int),
                ("exch_prob", ctypes.c_double), ("precision", ctypes.c_int),
                ("resync_every", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("cycles_per_launch", ctypes.c_int), ("device", ctypes.c_int)]


class Output(ctypes.Structure):
    _fields_ = [("en_avg", _dp), ("heat_cap", _dp), ("count_stat_atom", _dp),
                ("count_stat_vol", _dp), ("count_stat_exc", _dp), ("max_displ", _dp),
                ("en_histogram", _dp), ("ev_histogram", _dp),
                ("hist_params", ctypes.c_double * 6), ("rdf", _dp), ("delta_r2", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_launches", ctypes.c_longlong), ("graph_launches", ctypes.c_longlong),
                ("atom_moves", ctypes.c_longlong), ("volume_moves", ctypes.c_longlong),
                ("max_drift", ctypes.c_double), ("last_cycles_ms", ctypes.c_double)]


class SurrogateCfg(ctypes.Structure):
    _fields_ = [("r_lo", ctypes.c_double), ("r_hi", ctypes.c_double), ("gamma", ctypes.c_double),
                ("r_cut", ctypes.c_double), ("escale", ctypes.c_double)]


SUR_NPARAMS = 1633
_fp = ctypes.POINTER(ctypes.c_float)

# every symbol include/ptmc_gb300.h declares, with its ctypes signature
SIGNATURES = {
    "ptmc_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Params)]),
    "ptmc_set_potential_elj": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int]),
    "ptmc_set_potential_eam": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_double] * 4),
    "ptmc_set_potential_nn2": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, _dp, ctypes.c_int,
                                              _dp, _dp, ctypes.c_int, _ip, ctypes.c_int,
                                              ctypes.c_int]),
    "ptmc_set_atom_swaps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ptmc_get_swaps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _llp]),
    "ptmc_set_potential_eljb": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int]),
    "ptmc_set_potential_lookup": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int]
                                  + [ctypes.c_double] * 5),
    "ptmc_set_potential_nn": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int, _dp,
                                             ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double]),
    "ptmc_set_run_configs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "ptmc_set_run_configs_box": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_double]),
    "ptmc_set_runs_configs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double]),
    "ptmc_set_separated_volume": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ptmc_set_max_displ": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "ptmc_set_max_displ_sep": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "ptmc_set_rdf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ptmc_init": (ctypes.c_int, [ctypes.c_void_p]),
    "ptmc_equilibrate": (ctypes.c_int, [ctypes.c_void_p]),
    "ptmc_run_cycles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
    "ptmc_cycles_nosample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
    "ptmc_resync": (ctypes.c_int, [ctypes.c_void_p]),
    "ptmc_get_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Output)]),
    "ptmc_get_states": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp,
                                       _llp, _dp]),
    "ptmc_get_box_states": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _llp]),
    "ptmc_get_energies": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "ptmc_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "ptmc_checkpoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "ptmc_restore": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "ptmc_multihist_nvt": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          _dp, _dp, _ip]),
    "ptmc_multihist_npt": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          _dp, _dp, _ip]),
    "ptmc_multihist_nvt_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_double, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "ptmc_measure_peaks": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
    "ptmc_multihist_linear": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                             ctypes.c_double, ctypes.c_int, _dp, _dp, _ip, _dp, _dp,
                                             _dp, _dp, _dp, _dp, _dp]),
    "ptmc_surrogate_eval": (ctypes.c_int, [ctypes.POINTER(SurrogateCfg), _fp, _fp, ctypes.c_int,
                                           _dp, ctypes.c_int]),
    "ptmc_surrogate_loss_grad": (ctypes.c_int, [ctypes.POINTER(SurrogateCfg), _fp, _fp, _fp,
                                                ctypes.c_int, _dp, _fp, ctypes.c_int]),
    "ptmc_surrogate_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SurrogateCfg), _fp,
                                          ctypes.c_int, ctypes.c_int]),
    "ptmc_surrogate_record": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ptmc_surrogate_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, _dp]),
    "ptmc_surrogate_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "ptmc_surrogate_get": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.POINTER(SurrogateCfg),
                                          _llp]),
    "ptmc_surrogate_records": (ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int, _ip]),
    "ptmc_surrogate_calibrate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                                _dp]),
    "ptmc_surrogate_set_kappa": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "ptmc_set_launch_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int]),
    "ptmc_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, _ip]),
    "ptmc_set_wait_test": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int]),
    "ptmc_occupancy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip]),
    "ptmc_get_walker_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip]),
    "ptmc_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "ptmc_destroy": (None, [ctypes.c_void_p]),
    "ptmc_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path=LIB_PATH):
    """Load the engine library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libptmc_gb300.so is not built (%s); run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class PTMCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ptmc error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


def check(rc, ctx=None):
    if rc != PTMC_OK:
        raise PTMCError(rc, load().ptmc_last_error(ctx).decode(errors="replace"))
    return rc
