"""The C++ adapters (include/idpd/reference_api.hpp) as a reference host would
use them: tests/cpp/reference_api_run.cpp drives the reference's main-loop
body on an FDPS-style particle system through the adapters, then one
ChemManager event. Compared here with one oracle step from the same state
(the drift is bit-exact, forces within 1e-5) and with the same event run
directly through the C ABI.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, rel_force_err
from implicit_dpd_gb300 import build, configs
from implicit_dpd_gb300.abi import IdpdChemParams
from implicit_dpd_gb300.engine import LIB_PATH, Engine

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CORE = [0, 3]


def _compile(tmp):
    exe = os.path.join(tmp, "reference_api_run")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(build.nvcc())), "lib64")
    libdir = os.path.dirname(LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ps_standin"),
           os.path.join(ROOT, "tests", "cpp", "reference_api_run.cpp"), "-o", exe,
           "-L", libdir, "-lidpd_engine", "-Wl,-rpath," + libdir,
           "-L", cuda_lib, "-Wl,-rpath," + cuda_lib, "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _state():
    box = np.array([10.0, 10.0, 10.0])
    mem = configs.flat_bilayers(box, 600, seed=5, jitter=0.05)
    sol = configs.liquid(box, 1.0, seed=6)
    st = {k: np.concatenate([mem[k], sol[k]]) for k in ("pos", "vel", "acc", "prop", "amp_id", "unit")}
    n = len(st["pos"])
    st["id"] = np.arange(n, dtype=np.uint32)
    st["acc"] = np.random.default_rng(9).normal(0.0, 30.0, (n, 3))
    return box, st, 600


def _write_input(path, p, st, n_amp, cp, mt_seed, core_ptcl):
    n = len(st["pos"])
    with open(path, "wb") as f:
        f.write(bytes(p))
        np.array([n, n_amp, len(CORE)] + CORE, np.uint32).tofile(f)
        f.write(bytes(cp))
        np.array([mt_seed, len(core_ptcl)] + list(core_ptcl), np.uint32).tofile(f)
        rows = np.zeros(n, dtype=[("a", "<f8", 9), ("u", "<u4", 4)])
        rows["a"] = np.hstack([st["pos"], st["vel"], st["acc"]])
        rows["u"] = np.stack([st["id"], st["prop"], st["amp_id"], st["unit"]], 1)
        rows.tofile(f)


def _read_output(path, nsteps):
    b = open(path, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(b, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    n1 = int(take("<u4", 1)[0])
    rows = take("<f8", n1 * 24).reshape(n1, 24)
    out = {"pos": rows[:, 0:3], "vel": rows[:, 3:6], "acc": rows[:, 6:9], "dens": rows[:, 9:12],
           "press": rows[:, 12:15], "dsr": rows[:, 15:18], "nei_cm": rows[:, 18:24]}
    out["vir"] = take("<f8", 3 * nsteps).reshape(nsteps, 3)
    out["cont"] = int(take("<i4", 1)[0])
    out["amp_num"] = int(take("<u4", 1)[0])
    n2 = int(take("<u4", 1)[0])
    new = np.frombuffer(b, dtype=[("pos", "<f8", 3), ("vel", "<f8", 3), ("u", "<u4", 4)],
                        count=n2 - n1, offset=off)
    off += new.nbytes
    out["new"] = new
    nt = int(take("<u4", 1)[0])
    out["glob_topol"] = take("<u4", nt)
    return out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_adapters_drive_one_reference_step_and_an_event(tmp_path):
    exe = _compile(str(tmp_path))
    box, st, n_amp = _state()
    p = mdpd_params(box, time=99, cf_b_rigid=20.0)
    core_ptcl = [int(st["id"][(st["amp_id"] == a) & (st["unit"] == 0)][0]) for a in CORE]
    cp = IdpdChemParams(p_thresld=0.3, eps=0.2, influ_rad=2.0, influ_hei=0.8, influ_dep=4.0,
                        influ_grd=-0.5, amp_num=n_amp, max_amp_num=700)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, p, st, n_amp, cp, 1234, core_ptcl)
    subprocess.run([exe, inp, outp, "1"], check=True, timeout=300)
    out = _read_output(outp, 1)

    ref = {k: st[k].copy() for k in ("pos", "vel", "acc", "id", "prop")}
    ref["topol"], ref["cf_bend"] = O.build_topology(st["amp_id"], st["unit"], n_amp, CORE, p.cf_b,
                                                    p.cf_b_rigid)
    po = type(p).from_buffer_copy(p)
    O.md_step(po, ref, nthreads=4)
    assert np.array_equal(out["pos"], ref["pos"])
    assert np.array_equal(out["dsr"], ref["dsr"])
    assert rel_force_err(out["acc"], ref["acc"])[0] < FORCE_TOL
    f_rms = np.sqrt((ref["acc"] ** 2).sum(1).mean())
    assert np.abs(out["vel"] - ref["vel"]).max() < 0.5 * p.dt * FORCE_TOL * f_rms + 1e-12
    assert np.abs(out["dens"] - ref["dens"]).max() / np.abs(ref["dens"]).max() < FORCE_TOL
    assert np.abs(out["press"] - ref["press"]).max() / np.abs(ref["press"]).max() < 1e-4
    assert np.allclose(out["vir"][0], ref["bonded_vir"], rtol=1e-5)
    _, cm, _ = O.density(p, ref["pos"], ref["prop"], nthreads=4)
    ok = np.isfinite(cm)
    assert np.abs(out["nei_cm"][ok] - cm[ok]).max() < 1e-6  # FP32 cell-local sums

    # the event equals the same event through the C ABI on the same state
    e = Engine(sort_period=1000)
    q = type(p).from_buffer_copy(p)
    q.time = 100
    e.set_params(q)
    e.upload({"pos": out["pos"].copy(), "vel": out["vel"].copy(), "acc": out["acc"].copy(),
              "id": st["id"], "prop": st["prop"], "amp_id": st["amp_id"], "unit": st["unit"]})
    e.build_topology(n_amp, CORE)
    e.set_chem(cp, 1234, core_ptcl, 1024)
    cont = e.chem_event()
    d = e.download()
    n1 = len(out["pos"])
    assert out["cont"] == int(cont) and out["amp_num"] == e.chem_info()["amp_num"]
    assert len(out["new"]) == len(d["pos"]) - n1 > 0
    assert np.array_equal(out["new"]["pos"], d["pos"][n1:])
    assert np.array_equal(out["new"]["vel"], d["vel"][n1:])
    u = out["new"]["u"]
    for k, name in enumerate(("id", "prop", "amp_id", "unit")):
        assert np.array_equal(u[:, k], d[name][n1:]), name
    # glob_topol: the molecules' rows, new molecules appended
    gt = out["glob_topol"]
    assert len(gt) == 4 * out["amp_num"]
    assert np.array_equal(gt[4 * n_amp:], np.arange(n1, n1 + len(out["new"]), dtype=np.uint32))
