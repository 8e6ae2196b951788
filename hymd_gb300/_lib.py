"""ctypes binding of libhpf_gb300.so (the C ABI in include/hpf_gb300.h).

The shared library is the product: every numerical entry point of this package
goes through it.  There is no CPU or library fallback -- if the library is
missing or a CUDA device is absent, the call raises.
"""
import ctypes
import os
import re

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libhpf_gb300.so")
HEADER = os.path.join(ROOT, "include", "hpf_gb300.h")

HPF_REDUCE_BLOCKS = 1024
HPF_OUT_DOUBLES = 8 + 8 * HPF_REDUCE_BLOCKS + 8

STATUS = {
    0: "HPF_OK", 1: "HPF_ERR_ARG", 2: "HPF_ERR_CUDA", 3: "HPF_ERR_CUFFT",
    4: "HPF_ERR_INDEX", 5: "HPF_ERR_NONFINITE", 6: "HPF_ERR_TIMEOUT",
    7: "HPF_ERR_NOT_IMPLEMENTED", 8: "HPF_ERR_SCRATCH_LIMIT",
}


class HPFError(RuntimeError):
    def __init__(self, fn, code):
        self.code = code
        super().__init__(f"{fn} failed: {STATUS.get(code, code)}")


P = ctypes.c_void_p
I = ctypes.c_int
I64 = ctypes.c_int64
D = ctypes.c_double

_SIGNATURES = {
    "hpf_ctx_create": [ctypes.POINTER(P), I, I, I, I, ctypes.POINTER(D)],
    "hpf_ctx_destroy": [P],
    "hpf_ctx_set_box": [P, ctypes.POINTER(D), P],
    "hpf_ctx_box_state": [P, ctypes.POINTER(P)],
    "hpf_ctx_set_spectral": [P, I],
    "hpf_ctx_get_spectral": [P, ctypes.POINTER(I), ctypes.POINTER(I)],
    "hpf_topology_scratch_ints": [I64],  # returns int64 (restype set in lib())
    "hpf_topology_terms": [I64, I, P, P, P, P, P, P, I, P, I, P, I, P, P, P, I, P, P, P, P, P, P,
                           P, P, P],
    "hpf_ctx_set_spectral_tile": [P, I],
    "hpf_ctx_get_spectral_tile": [P, ctypes.POINTER(I), ctypes.POINTER(I)],
    "hpf_ctx_set_functional": [P, ctypes.POINTER(D), ctypes.POINTER(D), D, D],
    "hpf_get_error": [P, P, ctypes.POINTER(I)],
    "hpf_paint": [P, P, P, I64, ctypes.POINTER(D), P, P],
    "hpf_paint_charge": [P, P, P, I64, P, P],
    "hpf_r2c": [P, P, P, I, P],
    "hpf_c2r": [P, P, P, I, P],
    "hpf_kspace_force": [P, P, P, P, P, P, P],
    "hpf_kspace_sums": [P, P, P, ctypes.POINTER(D), P, P],
    "hpf_laplacian": [P, P, P, P],
    "hpf_energy_fp64": [P, P, P, I64, ctypes.POINTER(D), P, ctypes.POINTER(D), D, P, P],
    "hpf_readout": [P, P, P, P, I64, P, P],
    "hpf_bonds": [P, P, I64, P, P, P, P, P, I64, P, P, P],
    "hpf_angles": [P, P, I64, P, P, P, P, P, P, I64, P, P, P],
    "hpf_dihedrals": [P, P, I64, P, P, P, P, P, P, P, P, P, P, I64, I, P, P, P],
    "hpf_dipole_redistribute": [P, I64, P, P, P, P, P, P, P, P, I64, P],
    "hpf_kick": [P, ctypes.POINTER(P), I, I64, D, D, P],
    "hpf_inner_kick_drift": [P, P, P, P, P, I64, D, D, I, I, P, P],
    "hpf_respa_plan_create": [ctypes.POINTER(P), I64, I64, P, P, P, P, I64, P, P, P, P, P, I64,
                              P, P, P, P, P, P, P, I],
    "hpf_respa_plan_destroy": [P],
    "hpf_respa_plan_permute": [P, P, I64, P, I64, P, P],
    "hpf_respa_plan_counts": [P, ctypes.POINTER(I64), ctypes.POINTER(I64)],
    "hpf_respa_plan_info": [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)],
    "hpf_respa_step": [P, P, P, P, ctypes.POINTER(P), I, D, D, I, P, P, P, P, P, P, P, P, P,
                       P, P, P],
    "hpf_respa_step_paint": [P, P, P, P, ctypes.POINTER(P), I, D, D, I, P, P, P, P, P, P, P,
                             P, P, P, P, P, P, P],
    "hpf_sum_dot": [P, P, I64, P, P],
    "hpf_sum_v2": [P, I64, P, P],
}

class CsvrArgs(ctypes.Structure):
    """HpfCsvrArgs of include/hpf_gb300.h."""
    _fields_ = [("n_groups", I), ("remove_com", I), ("n_steps", I), ("stride", I),
                ("offset", I), ("advance", I), ("every", I), ("pad", I), ("count", D * 2),
                ("mass", D), ("gas_constant", D), ("target_temperature", D), ("c", D)]


class ScrArgs(ctypes.Structure):
    """HpfScrArgs of include/hpf_gb300.h."""
    _fields_ = [("n_types", I), ("n_steps", I), ("stride", I), ("advance", I), ("every", I),
                ("mode", I), ("couple_l", I), ("couple_n", I), ("half_mQm", D), ("mass", D),
                ("gas_constant", D), ("target_temperature", D), ("target_pressure", D),
                ("beta", D), ("tau_p", D), ("dt_outer", D), ("n_b", D),
                ("target_pressure_n", D)]


class Kick(ctypes.Structure):
    """HpfKick of include/hpf_gb300.h."""
    _fields_ = [("v", P), ("prev", P * 4), ("n_prev", I), ("pad", I), ("mass", D),
                ("dt_outer", D), ("thermo", ctypes.POINTER(CsvrArgs)), ("group", P),
                ("randoms", P), ("counter", P), ("state", P), ("ws", P), ("d_err", P)]


_SIGNATURES.update({
    "hpf_field_step": [P, P, P, I64, ctypes.POINTER(D), P, P, P, ctypes.POINTER(Kick), P],
    "hpf_pic_step": [P, P, P, I64, D, P, P, P, P, P, P, ctypes.POINTER(Kick), P],
    "hpf_pic_step_list": [P, P, P, P, I64, I64, D, P, P, ctypes.POINTER(Kick), P],
    "hpf_field_pic_step": [P, P, P, I64, ctypes.POINTER(D), P, P, P, P, P, I64, D, P, P,
                           ctypes.POINTER(Kick), I, P],
    "hpf_csvr_scale": [P, P, I64, P, I, P],
    "hpf_field_step_profile": [P, P, P, I64, ctypes.POINTER(D), P, P, P, ctypes.POINTER(Kick), P,
                               ctypes.POINTER(ctypes.c_float)],
    "hpf_csvr": [P, P, I64, ctypes.POINTER(P), I, D, ctypes.POINTER(CsvrArgs), P, P, P, P, P, P],
    "hpf_scr_isotropic": [P, P, P, I64, P, P, ctypes.POINTER(ScrArgs), P, P, P, P, P, P],
    "hpf_paint_static": [P, P, I64, I, I, I, I, ctypes.POINTER(D), ctypes.POINTER(D), P, P, P],
    "hpf_field_adjoint": [P, P, P, I64, ctypes.POINTER(D), P, P, P],
    "hpf_scr_scale_positions": [P, I64, P, I, P],
    "hpf_respa_forces": [P, P, P, P, P, P, P],
    "hpf_pic_force_vjp": [P, P, P, I64, D, P, P, P],
    "hpf_field_force_vjp": [P, P, P, I64, ctypes.POINTER(D), P, P, P, P],
    "hpf_dihedral_hvp": [P, P, P, I64, P, P, P, P, P, P, P, P, I64, P, P],
    "hpf_bonded_hvp": [P, P, P, I64, P, P, P, P, P, I64, P, P, P, P, P, I64, P, P],
    "hpf_gpe_step": [P, P, P, P, I64, P, ctypes.POINTER(D), ctypes.POINTER(D), D, D, D, I, I,
                     P, P, P, P, P, P, P, P, P, ctypes.POINTER(I), P],
})

_LIB = None


def header_symbols():
    """Names of every entry point declared in include/hpf_gb300.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\*)\s+(hpf_\w+)\s*\(", txt,
                                 re.M)))


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is not built; run `python -m hymd_gb300.build` "
                "(hymd_gb300 has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.hpf_topology_scratch_ints.restype = ctypes.c_int64
        L.hpf_status_string.argtypes = [ctypes.c_int]
        L.hpf_status_string.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def call(name, *args):
    code = getattr(lib(), name)(*args)
    if code != 0:
        raise HPFError(name, code)


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def dvec(vals):
    arr = (ctypes.c_double * len(vals))(*[float(v) for v in vals])
    return arr


def require_cuda(t, name, dtype=None, shape=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA torch.Tensor")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must have dtype {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} must have shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


def new_workspace(device=None):
    """Zeroed reduction workspace of HPF_OUT_DOUBLES doubles (results in [0:8])."""
    return torch.zeros(HPF_OUT_DOUBLES, dtype=torch.float64,
                       device=device if device is not None else "cuda")
