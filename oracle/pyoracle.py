"""ctypes front end of the CPU oracle (oracle/idpd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The library is built by
`make -C oracle` into oracle/_build/.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from implicit_dpd_gb300.abi import IdpdChemParams, IdpdParams, IdpdRunParam

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libidpd_oracle.so")
# the same restatement built with the reference's production flags
# (-O3 -ffast-math -funroll-loops, Makefile:10,21-23): CPU timing only
FAST_LIB_PATH = os.path.join(HERE, "_build", "libidpd_oracle_fast.so")

_lib = None

D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
U = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
I = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class OrcMT(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int32)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def use_fast_build(on):
    """Routes every wrapper below to the build with the reference's
    production flags (on) or back to the parity build (off). Timing only: the
    fast-math build is not a parity oracle."""
    global _lib
    _lib = _load(FAST_LIB_PATH if on else LIB_PATH)


def _load(path):
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.orc_saru_u32.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, U]
    L.orc_saru_nrml.restype = C.c_double
    L.orc_saru_nrml.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
    L.orc_mt_draws.argtypes = [C.c_uint32, C.c_int32, U]
    L.orc_mt_seed.argtypes = [C.POINTER(OrcMT), C.c_uint32]
    L.orc_derive_params.argtypes = [C.POINTER(IdpdRunParam), C.POINTER(IdpdParams)]
    L.orc_cells.restype = C.c_int32
    L.orc_cells.argtypes = [C.c_int32, D, D, C.c_double, I, I, I, I]
    L.orc_density.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, U, D, C.c_void_p,
                              C.c_void_p, C.c_int32]
    L.orc_force.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, D, U, U, D, D, C.c_void_p,
                            C.c_int32]
    L.orc_build_topology.argtypes = [C.c_int32, U, U, C.c_int32, C.c_int32, U, C.c_double,
                                     C.c_double, U, D]
    L.orc_bonded.argtypes = [C.POINTER(IdpdParams), C.c_int32, U, D, D, D, D]
    L.orc_drift.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, D, C.c_void_p, D, C.c_void_p]
    L.orc_kick.argtypes = [C.c_double, C.c_int32, D, D, D]
    L.orc_remove_cmdrift.argtypes = [C.c_int32, D]
    L.orc_md_step.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, D, D, D, D, U, U, C.c_int32,
                              C.c_void_p, C.c_void_p, D, D, D, C.c_int32]
    L.orc_chem_event.argtypes = [C.POINTER(IdpdParams), C.POINTER(IdpdChemParams),
                                 C.POINTER(OrcMT), C.POINTER(C.c_int32), C.c_int32, D, D, D, D,
                                 D, U, U, U, U, D, U, C.c_int32, U, C.POINTER(C.c_uint32),
                                 C.c_void_p, C.POINTER(C.c_int32)]
    L.orc_precursor.restype = C.c_int64
    L.orc_precursor.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, U, U, C.c_uint32,
                                C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.c_int32]
    L.orc_pairs_naive.restype = C.c_int64
    L.orc_pairs_naive.argtypes = [C.c_int32, D, D, C.c_double, U, U, C.c_int64]
    L.orc_pair_count.restype = C.c_int64
    L.orc_pair_count.argtypes = [C.POINTER(IdpdParams), C.c_int32, D, C.c_int32]
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def saru_u32(s1, s2, s3, count):
    out = np.zeros(count, np.uint32)
    lib().orc_saru_u32(s1, s2, s3, count, out)
    return out


def saru_nrml(s1, s2, s3):
    return lib().orc_saru_nrml(s1, s2, s3)


def mt_draws(seed, n):
    out = np.zeros(n, np.uint32)
    lib().orc_mt_draws(seed, n, out)
    return out


def derive_params(rp):
    out = IdpdParams()
    lib().orc_derive_params(C.byref(rp), C.byref(out))
    return out


def cells(pos, box, r_cell):
    n = len(pos)
    nc = np.zeros(3, np.int32)
    box = np.ascontiguousarray(box, np.float64)
    ncell_max = int(np.prod(np.floor(box / r_cell))) + 1
    cell_of = np.zeros(max(n, 1), np.int32)
    start = np.zeros(ncell_max + 1, np.int32)
    members = np.zeros(max(n, 1), np.int32)
    nce = lib().orc_cells(n, np.ascontiguousarray(pos), box, r_cell, nc, cell_of, start, members)
    if nce < 0:
        raise ValueError("box too small for the cell grid")
    return nc, cell_of[:n], start[: nce + 1], members[:n]


def density(p, pos, prop, nthreads=1, with_cm=True):
    n = len(pos)
    dens = np.zeros((n, 3))
    cm = np.zeros((n, 6)) if with_cm else None
    cnt = np.zeros((n, 2), np.uint32) if with_cm else None
    rc = lib().orc_density(C.byref(p), n, np.ascontiguousarray(pos), np.ascontiguousarray(prop,
                           np.uint32), dens, _ptr(cm), _ptr(cnt), nthreads)
    if rc != 0:
        raise ValueError("oracle density failed (box too small?)")
    return dens, cm, cnt


def force(p, pos, vel, pid, prop, dens, nthreads=1):
    n = len(pos)
    acc = np.zeros((n, 3))
    press = np.zeros((n, 3))
    rc = lib().orc_force(C.byref(p), n, np.ascontiguousarray(pos), np.ascontiguousarray(vel),
                         np.ascontiguousarray(pid, np.uint32), np.ascontiguousarray(prop, np.uint32),
                         np.ascontiguousarray(dens), acc, _ptr(press), nthreads)
    if rc != 0:
        raise ValueError("oracle force failed")
    return acc, press


def build_topology(amp_id, unit, n_amp, core_amp_id, cf_b, cf_b_rigid):
    topol = np.zeros(4 * max(n_amp, 1), np.uint32)
    cf_bend = np.zeros(max(n_amp, 1))
    core = np.ascontiguousarray(core_amp_id, np.uint32) if len(core_amp_id) else np.zeros(1, np.uint32)
    rc = lib().orc_build_topology(len(amp_id), np.ascontiguousarray(amp_id, np.uint32),
                                  np.ascontiguousarray(unit, np.uint32), n_amp, len(core_amp_id),
                                  core, cf_b, cf_b_rigid, topol, cf_bend)
    if rc != 0:
        raise ValueError("bad topology")
    return topol[: 4 * n_amp], cf_bend[:n_amp]


def bonded(p, topol, cf_bend, pos, acc):
    """acc += bonded forces (in place); returns the virial."""
    vir = np.zeros(3)
    n_amp = len(cf_bend)
    if n_amp == 0:
        return vir
    lib().orc_bonded(C.byref(p), n_amp, np.ascontiguousarray(topol, np.uint32),
                     np.ascontiguousarray(cf_bend), np.ascontiguousarray(pos), acc, vir)
    return vir


def drift(p, pos, vel, acc, dsr=None):
    """In place on pos/vel (and dsr); returns vel_buf."""
    vb = np.zeros_like(vel)
    lib().orc_drift(C.byref(p), len(pos), pos, vel, _ptr(vb), np.ascontiguousarray(acc), _ptr(dsr))
    return vb


def kick(dt, vel, vel_buf, acc):
    lib().orc_kick(dt, len(vel), vel, np.ascontiguousarray(vel_buf), np.ascontiguousarray(acc))


def remove_cmdrift(vel):
    lib().orc_remove_cmdrift(len(vel), vel)


def md_step(p, st, nthreads=1):
    """One main-loop iteration on the dict state `st` (updated in place)."""
    n = len(st["pos"])
    st.setdefault("dsr", np.zeros((n, 3)))
    vb = np.zeros((n, 3))
    dens = np.zeros((n, 3))
    press = np.zeros((n, 3))
    vir = np.zeros(3)
    topol = st.get("topol")
    cf_bend = st.get("cf_bend")
    n_amp = 0 if cf_bend is None else len(cf_bend)
    rc = lib().orc_md_step(C.byref(p), n, st["pos"], st["vel"], vb, st["acc"], st["dsr"],
                           np.ascontiguousarray(st["id"], np.uint32),
                           np.ascontiguousarray(st["prop"], np.uint32), n_amp,
                           _ptr(topol) if n_amp else None, _ptr(cf_bend) if n_amp else None,
                           dens, press, vir, nthreads)
    if rc != 0:
        raise ValueError("oracle step failed")
    st["dens"] = dens
    st["press"] = press
    st["bonded_vir"] = vir
    return st


def new_mt(seed):
    g = OrcMT()
    lib().orc_mt_seed(C.byref(g), seed)
    return g


def chem_event(p, cp, g, st, nei_cm, topol, core_ptcl_id, n_cap):
    """One RandomChemEvent; grows the arrays of the dict state `st`."""
    n0 = len(st["pos"])
    def grow(a, width):
        out = np.zeros((n_cap, width) if width else n_cap, a.dtype)
        out[:n0] = a
        return out
    pos, vel, acc = grow(st["pos"], 3), grow(st["vel"], 3), grow(st["acc"], 3)
    dsr = grow(st.get("dsr", np.zeros((n0, 3))), 3)
    vb = np.zeros((n_cap, 3))
    pid, prop = grow(st["id"], 0), grow(st["prop"], 0)
    amp_id, unit = grow(st["amp_id"], 0), grow(st["unit"], 0)
    n = C.c_int32(n0)
    amp_out = C.c_uint32(0)
    nt = C.c_int32(0)
    targets = np.zeros(2 * (1 << 20), np.uint32)
    core = np.ascontiguousarray(core_ptcl_id, np.uint32)
    rc = lib().orc_chem_event(C.byref(p), C.byref(cp), C.byref(g), C.byref(n), n_cap, pos, vel, vb,
                              acc, dsr, pid, prop, amp_id, unit, np.ascontiguousarray(nei_cm),
                              np.ascontiguousarray(topol, np.uint32), len(core), core,
                              C.byref(amp_out), targets.ctypes.data_as(C.c_void_p), C.byref(nt))
    if rc < 0:
        raise ValueError("chem capacity exceeded")
    m = n.value
    out = dict(st)
    out.update(pos=pos[:m], vel=vel[:m], acc=acc[:m], dsr=dsr[:m], id=pid[:m], prop=prop[:m],
               amp_id=amp_id[:m], unit=unit[:m])
    return rc, amp_out.value, targets[: 2 * nt.value].reshape(-1, 2), out


def precursor(p, pos, pid, prop, time, from_, near, to, threshold, seed, nthreads=1):
    """Precursor conversion (orc_precursor); returns (new prop, conversions)."""
    out = np.ascontiguousarray(prop, np.uint32).copy()
    cnt = lib().orc_precursor(C.byref(p), len(pos), np.ascontiguousarray(pos, np.float64),
                              np.ascontiguousarray(pid, np.uint32), out, time, from_, near, to,
                              threshold, seed, nthreads)
    if cnt < 0:
        raise ValueError("box too small for the cell grid")
    return out, int(cnt)


def pair_count(p, pos, nthreads=1):
    """Ordered pairs within the cutoff (r < 1, i != j)."""
    c = lib().orc_pair_count(C.byref(p), len(pos), np.ascontiguousarray(pos, np.float64), nthreads)
    if c < 0:
        raise ValueError("box too small for the cell grid")
    return int(c)


def pairs_naive(pos, box, rc=1.0):
    n = len(pos)
    cap = n * 64
    pi = np.zeros(cap, np.uint32)
    pj = np.zeros(cap, np.uint32)
    cnt = lib().orc_pairs_naive(n, np.ascontiguousarray(pos), np.ascontiguousarray(box, np.float64),
                                rc, pi, pj, cap)
    if cnt > cap:
        raise ValueError("pair capacity")
    return pi[:cnt], pj[:cnt]
