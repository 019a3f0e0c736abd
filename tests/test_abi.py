"""The C-ABI library loads and exports every symbol include/idpd_engine.h
declares; struct layouts agree between C and the ctypes mirrors; host-only
entry points work without a GPU."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import pyoracle as O
from implicit_dpd_gb300 import build as B
from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.abi import (IdpdChemConfig, IdpdChemInfo, IdpdChemParams, IdpdConfig,
                                    IdpdObservation, IdpdParams, IdpdPrecursor, IdpdRunParam,
                                    params_to_dict)
from implicit_dpd_gb300.engine import EXPORTS, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "idpd_engine.h")


@pytest.fixture(scope="module")
def lib():
    B.build()
    return load()


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(idpd_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(lib):
    decl = declared_symbols()
    assert set(decl) == set(EXPORTS), set(decl) ^ set(EXPORTS)
    for name in decl:
        assert hasattr(lib, name), name


def test_struct_layouts_match_c():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "idpd_engine.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(idpd_params), sizeof(idpd_run_param),
         sizeof(idpd_chem_params), sizeof(idpd_config), offsetof(idpd_params, seed),
         offsetof(idpd_params, cf_m), sizeof(idpd_chem_config),
         offsetof(idpd_chem_config, reserve_amp), sizeof(idpd_chem_info),
         offsetof(idpd_chem_info, core_raw), sizeof(idpd_observation),
         offsetof(idpd_observation, bonded_virial), sizeof(idpd_precursor),
         offsetof(idpd_precursor, enabled));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [int(x) for x in out]
    want = [C.sizeof(IdpdParams), C.sizeof(IdpdRunParam), C.sizeof(IdpdChemParams),
            C.sizeof(IdpdConfig), IdpdParams.seed.offset, IdpdParams.cf_m.offset,
            C.sizeof(IdpdChemConfig), IdpdChemConfig.reserve_amp.offset, C.sizeof(IdpdChemInfo),
            IdpdChemInfo.core_raw.offset, C.sizeof(IdpdObservation),
            IdpdObservation.bonded_virial.offset, C.sizeof(IdpdPrecursor),
            IdpdPrecursor.enabled.offset]
    assert got == want


def test_derive_params_c_abi_bit_exact_with_reference(lib):
    g = np.load(os.path.join(ROOT, "tests", "golden", "params.npz"))
    f32 = lambda x: float(np.float32(x))
    for k in range(int(g["n_sets"])):
        v = [f32(x) for x in g[f"{k}_input"]]
        rp = IdpdRunParam()
        for d in range(3):
            rp.box[d] = v[d]
        rp.dt = v[3]
        for q in range(6):
            rp.cf_r_upper[q] = v[4 + q]
        rp.cf_s, rp.cf_b, rp.cf_b_rigid, rp.vbb, rp.chi, rp.kappa, rp.rho_co = v[10:17]
        out = IdpdParams()
        assert lib.idpd_derive_params(C.byref(rp), C.byref(out)) == 0
        p = params_to_dict(out)
        for name in ("cf_c", "cf_g", "cf_r", "cf_m"):
            assert np.array_equal(p[name], g[f"{k}_{name}"]), (k, name)


def test_create_reports_missing_device_or_succeeds(lib):
    """Without a GPU the library answers with a status code, never aborts."""
    cfg = IdpdConfig(n_replicas=1)
    h = C.c_void_p()
    rc = lib.idpd_create(C.byref(cfg), C.byref(h))
    if rc == 0:
        lib.idpd_destroy(h)
    else:
        assert rc == 7  # IDPD_ERR_NO_DEVICE
        buf = C.create_string_buffer(256)
        lib.idpd_last_error(None, buf, 256)
        assert b"device" in buf.value


def test_invalid_arguments_are_rejected(lib):
    h = C.c_void_p()
    bad = IdpdConfig(n_replicas=0)
    assert lib.idpd_create(C.byref(bad), C.byref(h)) == 1
    assert lib.idpd_create(None, C.byref(h)) == 1


def test_cpp_adapters_compile_and_link(lib, tmp_path):
    """The C++ adapters (include/idpd/reference_api.hpp) compile against the
    reference's names (the FDPS stand-in of the oracle) as the adapter test's
    host program uses them, and link against the library; no GPU needed."""
    from implicit_dpd_gb300.engine import LIB_PATH
    exe = os.path.join(str(tmp_path), "reference_api_run")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(B.nvcc())), "lib64")
    libdir = os.path.dirname(LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ps_standin"),
           os.path.join(ROOT, "tests", "cpp", "reference_api_run.cpp"), "-o", exe,
           "-L", libdir, "-lidpd_engine", "-Wl,-rpath," + libdir,
           "-L", cuda_lib, "-Wl,-rpath," + cuda_lib, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(exe)


def test_host_saru_adapter_matches_reference_golden(tmp_path):
    """The host Saru of the C++ adapters against the golden draws of the
    reference's saruprng.hpp: u32() bit-exact, nrml() to FP64 rounding (the
    host libm's log and cos)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "saru.npz"))
    exe = os.path.join(str(tmp_path), "saru_host")
    subprocess.run(["g++", "-O2", "-std=c++11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "saru_host.cpp"), "-o", exe], check=True)
    seeds = g["seeds"]
    inp = "\n".join(f"{a} {b} {c}" for a, b, c in seeds) + "\n"
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout
    rows = [line.split() for line in out.strip().splitlines()]
    u = np.array([[int(x) for x in r[:4]] for r in rows], np.uint64).astype(np.uint32)
    nr = np.array([float(r[4]) for r in rows])
    assert np.array_equal(u, g["u32"][:, :4])
    assert np.abs(nr - g["nrml"]).max() < 1e-14 * max(1.0, np.abs(g["nrml"]).max())
