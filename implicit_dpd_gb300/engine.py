"""ctypes binding of the engine's C ABI (include/idpd_engine.h).

This is plumbing for tests and the benchmark; C and C++ callers link the
library directly (include/idpd/reference_api.hpp). The library is built
in-tree by implicit_dpd_gb300/build.py; loading fails loudly when it is
missing, there is no fallback path.
"""
import ctypes as C
import os

import numpy as np

from .abi import (STATUS_NAMES, IdpdChemConfig, IdpdChemInfo, IdpdConfig, IdpdObservation,
                  IdpdParams, IdpdPrecursor, IdpdRunFile, IdpdRunParam, IdpdTuning)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libidpd_engine.so")

D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
U = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
F = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
VP = C.c_void_p

# every symbol include/idpd_engine.h declares (tests/test_abi.py checks them)
EXPORTS = [
    "idpd_derive_params", "idpd_create", "idpd_destroy", "idpd_last_error", "idpd_set_params",
    "idpd_get_params", "idpd_upload_state", "idpd_num_particles", "idpd_download_state",
    "idpd_download_aux", "idpd_build_topology", "idpd_drift", "idpd_density", "idpd_force",
    "idpd_bonded", "idpd_kick", "idpd_remove_cmdrift", "idpd_step", "idpd_sync",
    "idpd_last_step_ms", "idpd_profile_step", "idpd_saru_u32", "idpd_saru_nrml_f32",
    "idpd_cell_order", "idpd_set_dynamics", "idpd_step_host", "idpd_set_tuning", "idpd_get_tuning",
    "idpd_cell_order_noalloc", "idpd_set_chem", "idpd_chem_event", "idpd_chem_get_info",
    "idpd_set_observe", "idpd_get_observations", "idpd_density_profile", "idpd_rdf",
    "idpd_dispatch_walks", "idpd_retrieve_walks", "idpd_read_run_param", "idpd_read_xyz",
    "idpd_write_xyz", "idpd_list_rebuilds", "idpd_set_precursor", "idpd_precursor_count",
    "idpd_pair_count", "idpd_dump_xyz_async", "idpd_dump_wait",
]

# The reference's EPI / EPJ / RESULT layouts (ptcl_class.hpp:5-174) as numpy
# record types, for the multi-walk interface.
WALK_DTYPES = {
    0: (np.dtype([("prop", "<u4"), ("pad", "<u4"), ("pos", "<f8", 3)]),
        np.dtype([("prop", "<u4"), ("pad", "<u4"), ("pos", "<f8", 3)]),
        np.dtype([("dens", "<f8", 3), ("nei_pos_sum", "<f8", (2, 3)), ("nei_cnt", "<u4", 2)])),
    1: (np.dtype([("id", "<u4"), ("prop", "<u4"), ("pos", "<f8", 3), ("vel", "<f8", 3),
                  ("dens", "<f8", 3)]),
        np.dtype([("id", "<u4"), ("prop", "<u4"), ("amp_id", "<u4"), ("unit", "<u4"),
                  ("pos", "<f8", 3), ("vel", "<f8", 3), ("dens", "<f8", 3)]),
        np.dtype([("acc", "<f8", 3), ("press", "<f8", 3)])),
}

_lib = None


class EngineError(RuntimeError):
    pass


def load(path=LIB_PATH):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise EngineError(f"engine library not built: {path} (run implicit_dpd_gb300.build)")
    L = C.CDLL(path)
    H = C.c_void_p
    L.idpd_derive_params.argtypes = [C.POINTER(IdpdRunParam), C.POINTER(IdpdParams)]
    L.idpd_create.argtypes = [C.POINTER(IdpdConfig), C.POINTER(H)]
    L.idpd_destroy.argtypes = [H]
    L.idpd_last_error.argtypes = [H, C.c_char_p, C.c_size_t]
    L.idpd_set_params.argtypes = [H, C.c_int32, C.POINTER(IdpdParams)]
    L.idpd_get_params.argtypes = [H, C.c_int32, C.POINTER(IdpdParams)]
    L.idpd_upload_state.argtypes = [H, C.c_int32, C.c_int32, D, D, VP, U, U, VP, VP]
    L.idpd_num_particles.argtypes = [H, C.c_int32, C.POINTER(C.c_int32)]
    L.idpd_download_state.argtypes = [H, C.c_int32, VP, VP, VP, VP, VP, VP, VP]
    L.idpd_download_aux.argtypes = [H, C.c_int32, VP, VP, VP, VP]
    L.idpd_build_topology.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, VP]
    for name in ("idpd_drift", "idpd_density", "idpd_force", "idpd_kick", "idpd_remove_cmdrift",
                 "idpd_sync"):
        getattr(L, name).argtypes = [H]
    L.idpd_bonded.argtypes = [H, VP]
    L.idpd_step.argtypes = [H, C.c_int32]
    L.idpd_last_step_ms.argtypes = [H, C.POINTER(C.c_float)]
    L.idpd_profile_step.argtypes = [H, C.c_char_p, C.c_size_t, F, C.c_int32, C.POINTER(C.c_int32)]
    L.idpd_saru_u32.argtypes = [C.c_int32, U, U, U, C.c_int32, U]
    L.idpd_saru_nrml_f32.argtypes = [C.c_int32, U, U, U, F]
    L.idpd_cell_order.argtypes = [H, C.c_int32, VP, VP]
    L.idpd_set_dynamics.argtypes = [H, C.c_int32, VP, VP, VP]
    L.idpd_step_host.argtypes = [H, C.c_int32, VP, VP, VP]
    L.idpd_set_tuning.argtypes = [H, C.POINTER(IdpdTuning)]
    L.idpd_get_tuning.argtypes = [H, C.POINTER(IdpdTuning)]
    L.idpd_list_rebuilds.argtypes = [H, C.POINTER(C.c_uint64)]
    L.idpd_pair_count.argtypes = [H, C.c_int32, C.POINTER(C.c_uint64)]
    L.idpd_dump_xyz_async.argtypes = [H, C.c_int32, C.c_char_p, C.c_int32]
    L.idpd_dump_wait.argtypes = [H]
    L.idpd_set_precursor.argtypes = [H, C.c_int32, C.POINTER(IdpdPrecursor)]
    L.idpd_precursor_count.argtypes = [H, C.c_int32, C.POINTER(C.c_uint64)]
    L.idpd_cell_order_noalloc.argtypes = [VP, C.c_int32, D, VP, VP, VP]
    L.idpd_set_chem.argtypes = [H, C.c_int32, C.POINTER(IdpdChemConfig)]
    L.idpd_chem_event.argtypes = [H, C.POINTER(C.c_int32)]
    L.idpd_chem_get_info.argtypes = [H, C.c_int32, C.POINTER(IdpdChemInfo), VP, C.c_int32]
    L.idpd_set_observe.argtypes = [H, C.c_int32, C.c_int32]
    L.idpd_get_observations.argtypes = [H, VP, C.c_int32, C.POINTER(C.c_int32)]
    L.idpd_density_profile.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, D]
    L.idpd_rdf.argtypes = [H, C.c_int32, C.c_int32, C.c_double, D]
    L.idpd_read_run_param.argtypes = [C.c_char_p, C.POINTER(IdpdRunFile)]
    L.idpd_read_xyz.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_int32),
                                C.POINTER(C.c_uint32), VP, VP, VP, VP, VP, VP, VP, VP]
    L.idpd_write_xyz.argtypes = [C.c_char_p, C.c_int32, C.c_uint32, C.c_int32, VP, VP, VP, VP,
                                 VP, VP, VP, VP]
    L.idpd_dispatch_walks.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, VP, VP, VP, VP]
    L.idpd_retrieve_walks.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, VP, VP]
    _lib = L
    return L


def _p(a):
    """Address of a numpy array, or of any buffer exposing data_ptr() (a torch
    tensor, page-locked or on the device)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def last_error(h=None):
    buf = C.create_string_buffer(512)
    load().idpd_last_error(h, buf, 512)
    return buf.value.decode()


def check(rc, h=None, what=""):
    if rc != 0:
        raise EngineError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {last_error(h)}")


def derive_params(rp):
    out = IdpdParams()
    check(load().idpd_derive_params(C.byref(rp), C.byref(out)), None, "derive_params")
    return out


def read_run_param(path):
    """run_param.txt as the reference's Parameter::LoadParam reads it."""
    out = IdpdRunFile()
    check(load().idpd_read_run_param(os.fsencode(path), C.byref(out)), None, "read_run_param")
    return out


def read_xyz(path, cap=None):
    """An xyz particle file: (state dict in the engine's upload form, time).
    cap defaults to the particle count of the header."""
    if cap is None:
        with open(path) as f:
            cap = int(f.readline())
    n = C.c_int32()
    t = C.c_uint32()
    st = {k: np.zeros((cap, 3)) for k in ("pos", "vel", "vel_buf", "acc")}
    for k in ("id", "prop", "amp_id", "unit"):
        st[k] = np.zeros(cap, np.uint32)
    check(load().idpd_read_xyz(os.fsencode(path), cap, C.byref(n), C.byref(t), _p(st["pos"]),
                               _p(st["vel"]), _p(st["vel_buf"]), _p(st["acc"]), _p(st["id"]),
                               _p(st["prop"]), _p(st["amp_id"]), _p(st["unit"])), None, "read_xyz")
    return {k: v[: n.value] for k, v in st.items()}, t.value


def write_xyz(path, st, time, append=False):
    """One frame in the reference's xyz format (vel_buf defaults to vel)."""
    n = len(st["pos"])
    a = {k: np.ascontiguousarray(st[k], np.float64) for k in ("pos", "vel", "acc")}
    vb = st.get("vel_buf")
    u = {k: np.ascontiguousarray(st[k], np.uint32) for k in ("id", "prop", "amp_id", "unit")}
    check(load().idpd_write_xyz(os.fsencode(path), int(append), time, n, _p(a["pos"]), _p(a["vel"]),
                                _p(None if vb is None else np.ascontiguousarray(vb, np.float64)),
                                _p(a["acc"]), _p(u["id"]), _p(u["prop"]), _p(u["amp_id"]),
                                _p(u["unit"])), None, "write_xyz")


def saru_u32(s1, s2, s3, draws):
    s1, s2, s3 = (np.ascontiguousarray(x, np.uint32) for x in (s1, s2, s3))
    out = np.zeros(len(s1) * draws, np.uint32)
    check(load().idpd_saru_u32(len(s1), s1, s2, s3, draws, out), None, "saru_u32")
    return out.reshape(len(s1), draws)


def saru_nrml_f32(s1, s2, s3):
    s1, s2, s3 = (np.ascontiguousarray(x, np.uint32) for x in (s1, s2, s3))
    out = np.zeros(len(s1), np.float32)
    check(load().idpd_saru_nrml_f32(len(s1), s1, s2, s3, out), None, "saru_nrml_f32")
    return out


class Engine:
    """One engine handle (idpd_handle*)."""

    def __init__(self, n_replicas=1, device=0, flags=0, sort_period=0, capacity=0):
        L = load()
        cfg = IdpdConfig(n_replicas=n_replicas, capacity=capacity, device=device, flags=flags,
                         sort_period=sort_period)
        h = C.c_void_p()
        check(L.idpd_create(C.byref(cfg), C.byref(h)), None, "idpd_create")
        self.h = h
        self.L = L
        self.R = n_replicas

    def close(self):
        if self.h:
            self.L.idpd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        check(rc, self.h, what)

    def set_params(self, p, replica=0):
        self._ck(self.L.idpd_set_params(self.h, replica, C.byref(p)), "set_params")

    def get_params(self, replica=0):
        p = IdpdParams()
        self._ck(self.L.idpd_get_params(self.h, replica, C.byref(p)), "get_params")
        return p

    def upload(self, st, replica=0):
        n = len(st["pos"])
        acc = st.get("acc")
        self._ck(self.L.idpd_upload_state(
            self.h, replica, n, np.ascontiguousarray(st["pos"], np.float64),
            np.ascontiguousarray(st["vel"], np.float64),
            _p(None if acc is None else np.ascontiguousarray(acc, np.float64)),
            np.ascontiguousarray(st["id"], np.uint32), np.ascontiguousarray(st["prop"], np.uint32),
            _p(np.ascontiguousarray(st["amp_id"], np.uint32)) if "amp_id" in st else None,
            _p(np.ascontiguousarray(st["unit"], np.uint32)) if "unit" in st else None), "upload")

    def set_dynamics(self, pos, vel, acc, replica=0):
        """pos/vel/acc: C-contiguous float64 (n, 3) arrays (pinned for speed)."""
        self._ck(self.L.idpd_set_dynamics(self.h, replica, _p(pos), _p(vel), _p(acc)),
                 "set_dynamics")

    def step_host(self, pos, vel, acc, replica=0):
        """One step on host (n, 3) float64 arrays, updated in place
        (idpd_step_host): set_dynamics + step(1) + download_dynamics in one call."""
        self._ck(self.L.idpd_step_host(self.h, replica, _p(pos), _p(vel), _p(acc)), "step_host")

    def download_dynamics(self, pos, vel, acc, replica=0):
        """Fills caller-provided (n, 3) float64 arrays, e.g. pinned buffers."""
        self._ck(self.L.idpd_download_state(self.h, replica, _p(pos), _p(vel), _p(acc), None, None,
                                            None, None), "download_dynamics")

    def set_chem(self, chem_params, mt_seed, core_ptcl_id, reserve_amp, beg_chem=100000,
                 replica=0):
        """ChemManager(mt_seed) with the Parameter values of chem_params
        (IdpdChemParams); None disables the reaction."""
        if chem_params is None:
            self._ck(self.L.idpd_set_chem(self.h, replica, None), "set_chem")
            return
        cfg = IdpdChemConfig(p=chem_params, mt_seed=mt_seed, beg_chem=beg_chem,
                             n_core=len(core_ptcl_id), reserve_amp=reserve_amp)
        for k, v in enumerate(core_ptcl_id):
            cfg.core_ptcl_id[k] = int(v)
        self._ck(self.L.idpd_set_chem(self.h, replica, C.byref(cfg)), "set_chem")

    def chem_event(self):
        """One RandomChemEvent; returns False when amp_num reached max_amp_num."""
        cont = C.c_int32()
        self._ck(self.L.idpd_chem_event(self.h, C.byref(cont)), "chem_event")
        return bool(cont.value)

    def chem_info(self, replica=0, max_targets=1 << 16):
        info = IdpdChemInfo()
        t = np.zeros(2 * max_targets, np.uint32)
        self._ck(self.L.idpd_chem_get_info(self.h, replica, C.byref(info), _p(t), max_targets),
                 "chem_info")
        nt = min(info.n_targets, max_targets)
        return {"n_targets": info.n_targets, "events": info.events, "stopped": bool(info.stopped),
                "amp_num": info.amp_num, "targets": t[: 2 * nt].reshape(-1, 2),
                "core_raw": np.array([list(r) for r in info.core_raw]),
                "h2t": np.array([list(r) for r in info.h2t])[: info.n_core],
                "core_h": np.array([list(r) for r in info.core_h])[: info.n_core]}

    def set_observe(self, period, capacity=4096):
        """Observer records every `period` steps (0: off)."""
        self._ck(self.L.idpd_set_observe(self.h, period, capacity), "set_observe")

    def observations(self, max_records=1 << 16):
        """Drains the recorded observations: a list of dicts, oldest first."""
        buf = (IdpdObservation * max_records)()
        n = C.c_int32()
        self._ck(self.L.idpd_get_observations(self.h, C.cast(buf, C.c_void_p), max_records,
                                              C.byref(n)), "observations")
        out = []
        for o in buf[: n.value]:
            out.append({"time": o.time, "replica": o.replica, "n": o.n, "n_amp": o.n_amp,
                        "kin_temp": np.array(o.kin_temp[:]), "pressure": np.array(o.pressure[:]),
                        "diffusion": np.array(o.diffusion[:]),
                        "pair_virial": np.array(o.pair_virial[:]),
                        "bonded_virial": np.array(o.bonded_virial[:])})
        return out

    def density_profile(self, axis=2, nbins=64, replica=0):
        out = np.zeros(3 * nbins)
        self._ck(self.L.idpd_density_profile(self.h, replica, axis, nbins, out), "density_profile")
        return out.reshape(nbins, 3)

    def rdf(self, nbins=100, r_max=2.0, replica=0):
        out = np.zeros(nbins)
        self._ck(self.L.idpd_rdf(self.h, replica, nbins, r_max, out), "rdf")
        return out

    def dispatch_walks(self, kind, epi, epj, tag=0):
        """DispatchKernel over walks: epi / epj are lists of record arrays of
        WALK_DTYPES[kind][0] / [1]."""
        n = len(epi)
        self._walk_keep = [np.ascontiguousarray(a) for a in epi] + [np.ascontiguousarray(a) for a in epj]
        pi = (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in self._walk_keep[:n]])
        pj = (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in self._walk_keep[n:]])
        ni = np.array([len(a) for a in epi], np.int32)
        nj = np.array([len(a) for a in epj], np.int32)
        self._walk_ni = ni
        self._ck(self.L.idpd_dispatch_walks(self.h, kind, tag, n, C.cast(pi, C.c_void_p), _p(ni),
                                            C.cast(pj, C.c_void_p), _p(nj)), "dispatch_walks")

    def retrieve_walks(self, kind, tag=0):
        """RetrieveKernel: one record array of WALK_DTYPES[kind][2] per walk."""
        ni = self._walk_ni
        out = [np.zeros(int(k), WALK_DTYPES[kind][2]) for k in ni]
        ptrs = (C.c_void_p * max(len(out), 1))(*[a.ctypes.data for a in out])
        self._ck(self.L.idpd_retrieve_walks(self.h, kind, tag, len(out), _p(ni),
                                            C.cast(ptrs, C.c_void_p)), "retrieve_walks")
        return out

    def set_tuning(self, reach, skin=None, lanes=None, blocks=None, dens_lanes=None):
        """reach 1 or 2; skin > 0 keeps the neighbour lists between rebuilds;
        lanes (4, 8, 16, 32) and blocks (1, 2, 4) shape the force pass,
        dens_lanes (4, 8, 16, 32) the density pass over kept lists (None: keep the current
        value)."""
        cur = IdpdTuning()
        self._ck(self.L.idpd_get_tuning(self.h, C.byref(cur)), "get_tuning")
        t = IdpdTuning(reach=reach, skin=cur.skin if skin is None else skin,
                       pair_lanes=cur.pair_lanes if lanes is None else lanes,
                       pair_blocks=cur.pair_blocks if blocks is None else blocks,
                       density_lanes=cur.density_lanes if dens_lanes is None else dens_lanes)
        self._ck(self.L.idpd_set_tuning(self.h, C.byref(t)), "set_tuning")

    def tuning(self):
        """The current tuning as a dict (reach, skin, lanes, blocks)."""
        t = IdpdTuning()
        self._ck(self.L.idpd_get_tuning(self.h, C.byref(t)), "get_tuning")
        return {"reach": t.reach, "skin": round(float(t.skin), 6), "lanes": t.pair_lanes,
                "blocks": t.pair_blocks, "dens_lanes": t.density_lanes}

    def set_precursor(self, prop_from, prop_near, prop_to, threshold, seed, replica=0,
                      enabled=True):
        """Precursor conversion of the replica (idpd_set_precursor); threshold is
        the u32 bound of the Saru draw (abi.precursor_threshold(p))."""
        cfg = IdpdPrecursor(prop_from=prop_from, prop_near=prop_near, prop_to=prop_to,
                            threshold=threshold, seed=seed, enabled=1 if enabled else 0)
        self._ck(self.L.idpd_set_precursor(self.h, replica, C.byref(cfg)), "set_precursor")

    def precursor_count(self, replica=0):
        n = C.c_uint64()
        self._ck(self.L.idpd_precursor_count(self.h, replica, C.byref(n)), "precursor_count")
        return n.value

    def list_rebuilds(self):
        """Steps that rebuilt the cells and kept lists (0 with skin 0)."""
        n = C.c_uint64()
        self._ck(self.L.idpd_list_rebuilds(self.h, C.byref(n)), "list_rebuilds")
        return n.value

    def dump_xyz_async(self, path, append=True, replica=0):
        """Queues a traject.xyz frame of the current state (written by a host
        thread while the steps go on)."""
        self._ck(self.L.idpd_dump_xyz_async(self.h, replica, os.fsencode(path), 1 if append else 0),
                 "dump_xyz_async")

    def dump_wait(self):
        """Blocks until the queued frame is written; raises on a failed frame."""
        self._ck(self.L.idpd_dump_wait(self.h), "dump_wait")

    def pair_count(self, replica=0):
        """Ordered pairs within the cutoff (r < 1) of the last density pass."""
        n = C.c_uint64()
        self._ck(self.L.idpd_pair_count(self.h, replica, C.byref(n)), "pair_count")
        return n.value

    def get_tuning(self):
        t = IdpdTuning()
        self._ck(self.L.idpd_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t.reach

    def get_skin(self):
        t = IdpdTuning()
        self._ck(self.L.idpd_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t.skin

    def num_particles(self, replica=0):
        n = C.c_int32()
        self._ck(self.L.idpd_num_particles(self.h, replica, C.byref(n)), "num_particles")
        return n.value

    def build_topology(self, n_amp, core_amp_id=(), replica=0):
        core = np.ascontiguousarray(list(core_amp_id) or [0], np.uint32)
        self._ck(self.L.idpd_build_topology(self.h, replica, n_amp, len(core_amp_id), _p(core)),
                 "build_topology")

    def download(self, replica=0):
        n = self.num_particles(replica)
        out = {k: np.zeros((n, 3)) for k in ("pos", "vel", "acc")}
        for k in ("id", "prop", "amp_id", "unit"):
            out[k] = np.zeros(n, np.uint32)
        self._ck(self.L.idpd_download_state(self.h, replica, _p(out["pos"]), _p(out["vel"]),
                                            _p(out["acc"]), _p(out["id"]), _p(out["prop"]),
                                            _p(out["amp_id"]), _p(out["unit"])), "download")
        return out

    def download_aux(self, replica=0, density=True, press=False, nei_cm=False, dsr=False):
        n = self.num_particles(replica)
        out = {}
        if density:
            out["dens"] = np.zeros((n, 3))
        if press:
            out["press"] = np.zeros((n, 3))
        if nei_cm:
            out["nei_cm"] = np.zeros((n, 6))
        if dsr:
            out["dsr"] = np.zeros((n, 3))
        self._ck(self.L.idpd_download_aux(self.h, replica, _p(out.get("dens")),
                                          _p(out.get("press")), _p(out.get("nei_cm")),
                                          _p(out.get("dsr"))), "download_aux")
        return out

    def drift(self):
        self._ck(self.L.idpd_drift(self.h), "drift")

    def density(self):
        self._ck(self.L.idpd_density(self.h), "density")

    def force(self):
        self._ck(self.L.idpd_force(self.h), "force")

    def bonded(self):
        vir = np.zeros(3 * self.R)
        self._ck(self.L.idpd_bonded(self.h, _p(vir)), "bonded")
        return vir.reshape(self.R, 3)

    def kick(self):
        self._ck(self.L.idpd_kick(self.h), "kick")

    def remove_cmdrift(self):
        self._ck(self.L.idpd_remove_cmdrift(self.h), "remove_cmdrift")

    def step(self, nsteps=1):
        self._ck(self.L.idpd_step(self.h, nsteps), "step")

    def sync(self):
        self._ck(self.L.idpd_sync(self.h), "sync")

    def last_step_ms(self):
        v = C.c_float()
        self._ck(self.L.idpd_last_step_ms(self.h, C.byref(v)), "last_step_ms")
        return v.value

    def profile_step(self):
        names = C.create_string_buffer(1024)
        ms = np.zeros(32, np.float32)
        nk = C.c_int32()
        self._ck(self.L.idpd_profile_step(self.h, names, 1024, ms, 32, C.byref(nk)), "profile_step")
        keys = names.value.decode().split()
        return dict(zip(keys, ms[: nk.value].tolist()))

    def cell_order(self, replica=0):
        n = self.num_particles(replica)
        cell = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        self._ck(self.L.idpd_cell_order(self.h, replica, _p(cell), _p(perm)), "cell_order")
        return cell, perm
