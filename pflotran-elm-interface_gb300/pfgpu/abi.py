"""ctypes mirror of include/pfgpu.h and the loader of the CUDA library.

The structs here are byte-for-byte the C structs of the public header; both
the GPU library (libpfgpu.so, built from ../csrc) and the CPU oracle take
them, so one host-side description drives both.
"""
from __future__ import annotations

import ctypes as C
import os

PF_OK = 0
PF_CELL_FAILURES = 1
PF_ERR_INVALID = -1
PF_ERR_UNSUPPORTED = -2
PF_ERR_CUDA = -3
PF_ERR_TOO_LARGE = -4
PF_ERR_TIMEOUT = -5

PF_CELL_OK = 0
PF_CELL_TOO_MANY_CUTS = 1
PF_CELL_NAN = 2
PF_CELL_NOT_RUN = -1

PF_ACT_COEF_OFF = 0
PF_ACT_COEF_TIMESTEP = 1
PF_ACT_COEF_NEWTON_ITER = 2
PF_ACT_COEF_ALGO_LAG = 0
PF_ACT_COEF_ALGO_NEWTON = 1

PF_KERNEL_PLAIN = 0
PF_KERNEL_BATCHED = 1

PF_BC_ZERO_FLUX = 0
PF_BC_DIRICHLET = 1
PF_BC_DIRICHLET_ZERO_GRADIENT = 2
PF_BC_ZERO_GRADIENT = 3
PF_SRC_VOLUMETRIC = 0
PF_SRC_EQUILIBRIUM = 1
PF_SRC_MASS_RATE = 2

PF_CONSTRAINT_TOTAL = 1
PF_CONSTRAINT_FREE = 2
PF_CONSTRAINT_PH = 3
PF_CONSTRAINT_CHARGE_BAL = 4
PF_CONSTRAINT_LOG = 5
PF_CONSTRAINT_MINERAL = 6
PF_CONSTRAINT_GAS = 7

PF_MAX_NCOMP = 24
PF_MAX_NSEC = 96
PF_MAX_NMNRL = 16
PF_MAX_SPEC_PER_RXN = 24
PF_MAX_NKD = 8
PF_MAX_NIONX = 4
PF_MAX_NSRFCPLX_RXN = 4
PF_MAX_NSRFCPLX = 16
PF_SURF_NULL = 0
PF_SURF_MINERAL = 1
PF_SURF_ROCK = 2
PF_MULTI_MAX_NETS = 16
PF_MAX_IONX_CATIONS = 8
PF_SORPTION_LINEAR = 1
PF_SORPTION_LANGMUIR = 2
PF_SORPTION_FREUNDLICH = 3
PF_KD_UNIT_KG_M3_BULK = 0
PF_KD_UNIT_MLW_GSOIL = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class PfOptions(C.Structure):
    _fields_ = [
        ("use_log_formulation", C.c_int32),
        ("act_coef_update_frequency", C.c_int32),
        ("act_coef_update_algorithm", C.c_int32),
        ("maximum_reaction_cuts", C.c_int32),
        ("maximum_reaction_iterations", C.c_int32),
        ("use_total_as_guess", C.c_int32),
        ("isothermal", C.c_int32),
        ("fork_literal_rsolve", C.c_int32),
        ("max_dlnC_rreact", C.c_double),
        ("max_relative_change_tolerance", C.c_double),
        ("max_residual_tolerance", C.c_double),
        ("max_rel_residual_tolerance", C.c_double),
        ("use_activity_h2o", C.c_int32),
    ]


class PfSorptionDesc(C.Structure):
    _fields_ = [
        ("nkd", C.c_int32), ("kd_units", C.c_int32),
        ("kd_spec", _ip), ("kd_type", _ip), ("kd_coeff", _dp), ("kd_langmuir_b", _dp),
        ("kd_freundlich_n", _dp), ("kd_mineral", _ip), ("soil_particle_density", C.c_double),
        ("nionx", C.c_int32), ("ionx_stride", C.c_int32),
        ("ionx_ncation", _ip), ("ionx_cation", _ip), ("ionx_k", _dp), ("ionx_cec", _dp), ("ionx_mineral", _ip),
        ("nsrfcplx_rxn", C.c_int32), ("nsrfcplx", C.c_int32), ("srfcplx_rxn_ptr", _ip), ("srfcplx_surf_type", _ip),
        ("srfcplx_mineral", _ip), ("srfcplx_site_density", _dp), ("srfcplx_stride", C.c_int32),
        ("srfcplx_nspec", _ip), ("srfcplx_spec", _ip), ("srfcplx_stoich", _dp), ("srfcplx_free_site_stoich", _dp),
        ("srfcplx_logK", _dp), ("srfcplx_logKcoef", _dp), ("srfcplx_h2o_stoich", _dp),
    ]


PF_MAX_PREFACTORS = 4
PF_MAX_PREFACTOR_SPECIES = 4


class PfPrefactorDesc(C.Structure):
    _fields_ = [
        ("num_prefactors", _ip), ("rate", _dp), ("activation_energy", _dp), ("nspec", _ip), ("spec", _ip),
        ("alpha", _dp), ("beta", _dp), ("atten_coef", _dp),
    ]


class PfNetworkDesc(C.Structure):
    _fields_ = [
        ("ncomp", C.c_int32), ("nsec", C.c_int32), ("nmnrl", C.c_int32),
        ("sec_stride", C.c_int32), ("mnrl_stride", C.c_int32), ("h_ion_id", C.c_int32),
        ("sec_nspec", _ip), ("sec_spec", _ip), ("sec_stoich", _dp),
        ("sec_logK", _dp), ("sec_logKcoef", _dp),
        ("pri_Z", _dp), ("pri_a0", _dp), ("sec_Z", _dp), ("sec_a0", _dp),
        ("mnrl_nspec", _ip), ("mnrl_spec", _ip), ("mnrl_stoich", _dp),
        ("mnrl_logK", _dp), ("mnrl_logKcoef", _dp),
        ("mnrl_rate_constant", _dp), ("mnrl_activation_energy", _dp),
        ("mnrl_molar_vol", _dp), ("mnrl_affinity_threshold", _dp),
        ("mnrl_rate_limiter", _dp), ("mnrl_irreversible", _ip),
        ("mnrl_min_scale_factor", _dp), ("mnrl_Temkin_const", _dp),
        ("mnrl_affinity_power", _dp),
        ("debyeA", C.c_double), ("debyeB", C.c_double), ("debyeBdot", C.c_double),
        ("opts", PfOptions),
        ("sorption", C.POINTER(PfSorptionDesc)),
        ("prefactors", C.POINTER(PfPrefactorDesc)),
        ("sec_h2o_stoich", _dp), ("mnrl_h2o_stoich", _dp),
    ]


class PfCellState(C.Structure):
    _fields_ = [
        ("ncells", C.c_int64),
        ("total", _dp), ("pri_molal", _dp), ("pri_act_coef", _dp),
        ("sec_act_coef", _dp), ("sec_molal", _dp),
        ("mnrl_volfrac", _dp), ("mnrl_area", _dp), ("mnrl_rate", _dp),
        ("porosity", _dp), ("saturation", _dp), ("den_kg", _dp),
        ("volume", _dp), ("temperature", _dp), ("dt_cell", _dp),
        ("status", _ip), ("newton_its", _ip), ("num_substeps", _ip),
        ("cell_order", C.POINTER(C.c_int64)),
        ("total_sorb", _dp), ("ionx_ref_sorbed", _dp), ("ln_act_h2o", _dp),
        ("srfcplx_free_site", _dp), ("srfcplx_conc", _dp),
    ]


class PfStepStats(C.Structure):
    _fields_ = [
        ("cells", C.c_int64), ("failed_cells", C.c_int64),
        ("newton_iterations", C.c_int64),
        ("max_newton_iterations", C.c_int32), ("max_substeps", C.c_int32),
    ]


PF_ADJ_MAX_SUBSTEPS = 16


class PfAdjointArgs(C.Structure):
    _fields_ = [
        ("weight", _dp), ("target", _dp), ("dL_dtotal", _dp), ("dL_dtotal0", _dp),
        ("dL_dlnarea", _dp), ("dL_dlogK_sec", _dp), ("dL_dlogK_mnrl", _dp), ("dL_dlnk", _dp),
        ("loss", _dp), ("adj_status", _ip),
    ]


class PfGirtArgs(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("qx", _dp), ("qy", _dp), ("qz", _dp),
        ("diffusion_coefficient", C.c_double), ("tortuosity", C.c_double), ("dispersivity", C.c_double),
        ("total_k", _dp), ("dt", C.c_double), ("rowptr", _ip), ("colidx", _ip),
        ("residual", _dp), ("values", _dp), ("total_sorb_k", _dp), ("numerical_derivatives", C.c_int32),
        ("k_cache", _dp), ("k_cache_valid", C.c_int32),
    ]


class PfTransportArgs(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("ncomp", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("qx", _dp), ("qy", _dp), ("qz", _dp),
        ("diffusion_coefficient", C.c_double), ("tortuosity", C.c_double), ("dispersivity", C.c_double),
        ("porosity", _dp), ("saturation", _dp), ("volume", _dp),
        ("dt", C.c_double), ("total", _dp), ("rtol", C.c_double), ("max_iterations", C.c_int32),
        ("bc_type", C.c_int32 * 6), ("bc_q", _dp * 6), ("bc_total", _dp * 6), ("bc_saturation", C.c_double * 6),
        ("nsrc", C.c_int32), ("src_cell", C.POINTER(C.c_int32)), ("src_type", C.POINTER(C.c_int32)),
        ("src_q", _dp), ("src_total", _dp),
    ]


class PfTransportStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("max_rel_residual", C.c_double),
                ("refinements", C.c_int32), ("max_cycle_iterations", C.c_int32)]


class PfConstraintReaction(C.Structure):
    _fields_ = [("nspec", C.c_int32), ("temperature_dependent", C.c_int32),
                ("spec", C.c_int32 * PF_MAX_NCOMP), ("stoich", C.c_double * PF_MAX_NCOMP),
                ("logK", C.c_double), ("logKcoef", C.c_double * 5)]


def constraint_reactions(ncomp: int, reactions):
    """A PfConstraintReaction array [ncomp] from {component index: dict(spec=
    [primary indices], stoich=[...], logK=..., logKcoef=[5] or None)} (the
    MINERAL/GAS rows; other entries stay empty).  Returns None for no
    reactions."""
    if not reactions:
        return None
    arr = (PfConstraintReaction * ncomp)()
    for j, r in reactions.items():
        e = arr[int(j)]
        spec, stoich = list(r["spec"]), list(r["stoich"])
        if not 1 <= len(spec) <= ncomp or len(spec) != len(stoich):
            raise ValueError("constraint reaction of component %d: bad species list" % j)
        e.nspec = len(spec)
        for p, (k, nu) in enumerate(zip(spec, stoich)):
            e.spec[p], e.stoich[p] = int(k), float(nu)
        e.logK = float(r["logK"])
        coef = r.get("logKcoef")
        e.temperature_dependent = 1 if coef is not None else 0
        if coef is not None:
            for p in range(5):
                e.logKcoef[p] = float(coef[p])
    return arr


class PfLaunchConfig(C.Structure):
    _fields_ = [
        ("threads_per_block", C.c_int32), ("blocks_per_sm", C.c_int32),
        ("jac_in_shared", C.c_int32), ("lanes_per_cell", C.c_int32),
    ]


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libpfgpu.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

# Every exported symbol with its ctypes signature (restype, argtypes).
_P = C.c_void_p
SIGNATURES = {
    "pf_network_create": (C.c_int32, [C.POINTER(PfNetworkDesc), C.POINTER(_P)]),
    "pf_network_destroy": (C.c_int32, [_P]),
    "pf_network_set_options": (C.c_int32, [_P, C.POINTER(PfOptions)]),
    "pf_network_reserve": (C.c_int32, [_P, C.c_int64]),
    "pf_rstep": (C.c_int32, [_P, C.POINTER(PfCellState), C.c_double, C.c_int32, _P,
                             C.POINTER(PfStepStats)]),
    "pf_update_auxvars": (C.c_int32, [_P, C.POINTER(PfCellState), C.c_int32, _P]),
    "pf_update_activity_coefs": (C.c_int32, [_P, C.POINTER(PfCellState), _P]),
    "pf_adjoint": (C.c_int32, [_P, C.POINTER(PfCellState), C.c_double, C.POINTER(PfAdjointArgs), _P]),
    "pf_network_shift_parameters": (C.c_int32, [_P, _dp, _dp, _dp]),
    "pf_girt_pattern": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, _ip, _ip]),
    "pf_transport_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.POINTER(_P)]),
    "pf_transport_destroy": (C.c_int32, [_P]),
    "pf_transport_step": (C.c_int32, [_P, C.POINTER(PfTransportArgs), _P, C.POINTER(PfTransportStats)]),
    "pf_transport_enqueue": (C.c_int32, [_P, C.POINTER(PfTransportArgs), C.c_int32, C.c_int32, _P]),
    "pf_transport_read_stats": (C.c_int32, [_P, C.c_double, _P, C.POINTER(PfTransportStats)]),
    "pf_girt_assemble": (C.c_int32, [_P, C.POINTER(PfCellState), C.POINTER(PfGirtArgs), _P]),
    "pf_rstep_noalloc": (C.c_int32, [_P, C.POINTER(PfCellState), C.c_double, _P, C.POINTER(PfStepStats)]),
    "pf_rstep_multi": (C.c_int32, [C.POINTER(C.c_void_p), C.POINTER(PfCellState), C.c_int32, C.c_double, _P,
                                   C.POINTER(PfStepStats)]),
    "pf_rstep_host": (C.c_int32, [_P, C.POINTER(PfCellState), C.c_double, C.c_int32,
                                  C.POINTER(PfStepStats)]),
    "pf_equilibrate_constraint": (C.c_int32, [_P, C.POINTER(PfCellState), C.POINTER(C.c_int32),
                                              _P, C.c_int32, _P, _P]),
    "pf_equilibrate_constraint_ex": (C.c_int32, [_P, C.POINTER(PfCellState), C.POINTER(C.c_int32), _P,
                                                 _P, C.c_int32, _P, _P]),
    "pf_network_set_launch": (C.c_int32, [_P, C.POINTER(PfLaunchConfig)]),
    "pf_network_get_launch": (C.c_int32, [_P, C.POINTER(PfLaunchConfig)]),
    "pf_version": (C.c_char_p, []),
    "pf_bench_fp64_fma": (C.c_int32, [_P, C.c_int64, C.c_int32, C.c_int32, _P]),
}

_lib = None


class PfError(RuntimeError):
    def __init__(self, fn, code):
        super().__init__(f"{fn} returned {code}")
        self.code = code


def load(path: str | None = None):
    """Load libpfgpu.so (built in-tree by __graft_entry__.build()).

    Raises if the library is missing: there is no fallback path.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} not found: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(fn: str, code: int, allow_cell_failures: bool = True) -> int:
    if code == PF_OK or (allow_cell_failures and code == PF_CELL_FAILURES):
        return code
    raise PfError(fn, code)
