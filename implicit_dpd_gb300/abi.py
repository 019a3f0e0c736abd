"""ctypes mirrors of the plain-C structs declared in include/idpd_engine.h.

The layouts must match the header field for field; tests/test_abi.py checks the
sizes against the compiled library.
"""
import ctypes as C

HYPHIL, HYPHOB, SOLVENT = 0, 1, 2  # parameter.hpp:208-214
FORM_MDPD, FORM_PAIRWISE, FORM_WARREN = 0, 1, 2

OK = 0
STATUS_NAMES = {
    0: "IDPD_OK",
    1: "IDPD_ERR_INVALID_ARG",
    2: "IDPD_ERR_CAPACITY",
    3: "IDPD_ERR_CUDA",
    4: "IDPD_ERR_TIMEOUT",
    5: "IDPD_ERR_NONFINITE",
    6: "IDPD_ERR_STATE",
    7: "IDPD_ERR_NO_DEVICE",
}

CFG_FP64_PAIRS = 0x1
CFG_FP64_KEPT = 0x4
CFG_TIMING = 0x2
CFG_PLAIN_GRAPHS = 0x8  # one graph launch per step, no conditional nodes (same results)

NONE32 = 0xFFFFFFFF  # amp_id / unit of solvent beads (parameter.hpp:450-451)


class IdpdParams(C.Structure):
    _fields_ = [
        ("box", C.c_double * 3),
        ("dt", C.c_double),
        ("cf_c", (C.c_double * 3) * 3),
        ("cf_g", (C.c_double * 3) * 3),
        ("cf_r", (C.c_double * 3) * 3),
        ("cf_m", ((C.c_double * 3) * 3) * 3),
        ("cf_s", C.c_double),
        ("cf_b", C.c_double),
        ("cf_b_rigid", C.c_double),
        ("warren_a", C.c_double),
        ("warren_b", C.c_double),
        ("warren_rd", C.c_double),
        ("seed", C.c_uint32),
        ("time", C.c_uint32),
        ("form", C.c_int32),
        ("reserved", C.c_int32),
    ]


class IdpdRunParam(C.Structure):
    _fields_ = [
        ("box", C.c_double * 3),
        ("dt", C.c_double),
        ("cf_r_upper", C.c_double * 6),
        ("cf_s", C.c_double),
        ("cf_b", C.c_double),
        ("cf_b_rigid", C.c_double),
        ("vbb", C.c_double),
        ("chi", C.c_double),
        ("kappa", C.c_double),
        ("rho_co", C.c_double),
    ]


class IdpdChemParams(C.Structure):
    _fields_ = [
        ("p_thresld", C.c_double),
        ("eps", C.c_double),
        ("influ_rad", C.c_double),
        ("influ_hei", C.c_double),
        ("influ_dep", C.c_double),
        ("influ_grd", C.c_double),
        ("amp_num", C.c_uint32),
        ("max_amp_num", C.c_uint32),
    ]


CHEM_MAX_CORE = 8
WALK_DENSITY, WALK_FORCE = 0, 1


class IdpdChemConfig(C.Structure):
    _fields_ = [
        ("p", IdpdChemParams),
        ("mt_seed", C.c_uint32),
        ("beg_chem", C.c_uint32),
        ("n_core", C.c_int32),
        ("core_ptcl_id", C.c_uint32 * CHEM_MAX_CORE),
        ("reserve_amp", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class IdpdRunFile(C.Structure):
    _fields_ = [
        ("rp", IdpdRunParam),
        ("init_amp_num", C.c_uint32),
        ("sol_num", C.c_uint32),
        ("all_time", C.c_uint32),
        ("step_mic", C.c_uint32),
        ("step_mac", C.c_uint32),
        ("has_chem", C.c_int32),
        ("chem", IdpdChemParams),
        ("influ_vol", C.c_double),
        ("upside_rad", C.c_double),
        ("n_core", C.c_int32),
        ("core_amp_id", C.c_uint32 * CHEM_MAX_CORE),
    ]


class IdpdObservation(C.Structure):
    _fields_ = [
        ("time", C.c_uint32),
        ("replica", C.c_int32),
        ("n", C.c_int32),
        ("n_amp", C.c_int32),
        ("kin_temp", C.c_double * 4),
        ("pressure", C.c_double * 3),
        ("diffusion", C.c_double * 3),
        ("pair_virial", C.c_double * 3),
        ("bonded_virial", C.c_double * 3),
    ]


class IdpdChemInfo(C.Structure):
    _fields_ = [
        ("n_targets", C.c_int32),
        ("events", C.c_int32),
        ("stopped", C.c_int32),
        ("amp_num", C.c_uint32),
        ("core_raw", (C.c_double * 9) * CHEM_MAX_CORE),
        ("n_core", C.c_int32),
        ("reserved", C.c_int32),
        ("h2t", (C.c_double * 3) * CHEM_MAX_CORE),
        ("core_h", (C.c_double * 3) * CHEM_MAX_CORE),
    ]


class IdpdConfig(C.Structure):
    _fields_ = [
        ("n_replicas", C.c_int32),
        ("capacity", C.c_int32),
        ("device", C.c_int32),
        ("flags", C.c_int32),
        ("sort_period", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class IdpdTuning(C.Structure):
    _fields_ = [("reach", C.c_int32), ("skin", C.c_float), ("pair_lanes", C.c_int32),
                ("pair_blocks", C.c_int32), ("density_lanes", C.c_int32),
                ("reserved", C.c_int32 * 3)]


class IdpdPrecursor(C.Structure):
    _fields_ = [("prop_from", C.c_uint32), ("prop_near", C.c_uint32), ("prop_to", C.c_uint32),
                ("threshold", C.c_uint32), ("seed", C.c_uint32), ("enabled", C.c_int32),
                ("reserved", C.c_int32 * 2)]


def precursor_threshold(p):
    """The u32 threshold of a conversion probability p per step: floor(p 2^32)."""
    return min(int(p * 4294967296.0), 0xFFFFFFFF)


def params_to_dict(p):
    import numpy as np

    return {
        "box": np.array(p.box[:]),
        "dt": p.dt,
        "cf_c": np.ctypeslib.as_array(p.cf_c).copy(),
        "cf_g": np.ctypeslib.as_array(p.cf_g).copy(),
        "cf_r": np.ctypeslib.as_array(p.cf_r).copy(),
        "cf_m": np.ctypeslib.as_array(p.cf_m).copy(),
        "cf_s": p.cf_s,
        "cf_b": p.cf_b,
        "cf_b_rigid": p.cf_b_rigid,
        "seed": p.seed,
        "time": p.time,
        "form": p.form,
    }


def f32(x):
    """Round a Python float through binary32, as std::stof does when the
    reference parses run_param.txt (parameter.hpp:339)."""
    import numpy as np

    return float(np.float32(x))
