"""On-disk formats and configuration shapes (host code, no GPU):

* run_param.txt through the engine library's reader (Parameter::LoadParam
  semantics: ';' comments, std::stof rounding, required tags, the influence
  cone from influ_vol + upside_rad or from influ_rad + influ_grd);
* xyz frames written and read back in the reference's row format;
* flat, spherical and cylindrical bilayers with the config maker's geometry.
"""
import os

import numpy as np
import pytest

from implicit_dpd_gb300 import configs
from implicit_dpd_gb300.engine import EngineError, read_run_param, read_xyz, write_xyz

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUN = """; run input
box_leng 35.0 35.0 28.1   ; box
init_amp_num 4680
sol_num 12
dt 0.005
cf_r 3.0 3.0 3.0 3.0 3.0 3.0
cf_s 19.0
cf_b 5.0
cf_b_rigid 7.3
chi 30.0
kappa 100.0
rho_co 17.0
all_time 40000
step_mic 5000
step_mac 1
p_thresld 0.001
eps 0.2
max_amp_num 9000
influ_hei 0.8
influ_dep 4.1
{cone}
core_amp_id 3 11
"""


def _lib_built():
    from implicit_dpd_gb300.engine import LIB_PATH
    return os.path.exists(LIB_PATH)


pytestmark = pytest.mark.skipif(not _lib_built(), reason="engine library not built")


def test_run_param_stof_rounding_and_cone_from_radius(tmp_path):
    f = tmp_path / "run_param.txt"
    f.write_text(RUN.format(cone="influ_rad 2.1\ninflu_grd -0.3"))
    r = read_run_param(str(f))
    f32 = lambda v: float(np.float32(v))
    assert list(r.rp.box) == [35.0, 35.0, f32(28.1)]
    assert r.rp.dt == f32(0.005) and r.rp.cf_b_rigid == f32(7.3) and r.rp.vbb == pytest.approx(0.1)
    assert (r.init_amp_num, r.sol_num, r.all_time, r.step_mic, r.step_mac) == (4680, 12, 40000, 5000, 1)
    assert r.has_chem == 1 and r.n_core == 2 and list(r.core_amp_id[:2]) == [3, 11]
    c = r.chem
    assert (c.p_thresld, c.influ_rad, c.influ_grd) == (f32(0.001), f32(2.1), f32(-0.3))
    assert c.amp_num == 4680 and c.max_amp_num == 9000
    # CalcInfluVol, parameter.hpp:58-72 (truncated cone)
    hs = c.influ_hei + c.influ_dep
    up, down = c.influ_rad - c.influ_grd * c.influ_hei, c.influ_rad + c.influ_grd * c.influ_dep
    ua, da = np.pi * up * up, np.pi * down * down
    assert r.influ_vol == pytest.approx((ua + da + np.sqrt(ua * da)) * hs / 3.0, rel=1e-15)


def test_run_param_cone_from_volume(tmp_path):
    f = tmp_path / "run_param.txt"
    f.write_text(RUN.format(cone="influ_vol 40.0\nupside_rad 1.5"))
    r = read_run_param(str(f))
    c = r.chem
    hs = c.influ_hei + c.influ_dep
    up = r.upside_rad
    val = 12.0 * r.influ_vol / (np.pi * hs) - 3.0 * up * up
    grd = ((np.sqrt(val) - up) * 0.5 - up) / hs
    assert c.influ_grd == pytest.approx(grd, rel=1e-15)
    assert c.influ_rad == pytest.approx(up + grd * c.influ_hei, rel=1e-15)


def test_run_param_missing_tag_is_named(tmp_path):
    f = tmp_path / "run_param.txt"
    f.write_text(RUN.format(cone="").replace("kappa 100.0\n", ""))
    with pytest.raises(EngineError, match="kappa"):
        read_run_param(str(f))


def test_reference_profile_input_lacks_required_tags(tmp_path):
    """profile/test_result/omp1/run_param.txt of the reference predates
    cf_b_rigid and the reaction tags; LoadParam would abort on it."""
    text = ("box_leng 35.0 35.0 35.0\ninit_amp_num 4680\ndt 0.005\ncf_r 3.0 3.0 3.0\n"
            "cf_s 19.0\ncf_b 5.0\nrc 1.0\nchi 30.0\nkappa 100.0\nrho_co 17.0\nall_time 40000\n"
            "step_mac 1\nstep_mic 5000\nTemperature 1.0\n")
    f = tmp_path / "run_param.txt"
    f.write_text(text)
    with pytest.raises(EngineError, match="sol_num"):
        read_run_param(str(f))


def test_xyz_round_trip_in_the_reference_row_format(tmp_path):
    st = configs.flat_bilayers(np.array([6.0, 6.0, 6.0]), 50, seed=3)
    st["acc"] = np.random.default_rng(1).normal(size=st["pos"].shape)
    f = tmp_path / "traject.xyz"
    write_xyz(str(f), st, 123)
    lines = f.read_text().splitlines()
    assert lines[0] == str(len(st["pos"])) and lines[1] == "time 123"
    head = lines[2].split()
    assert head[0] == "O" and lines[3].split()[0] == "N"  # Hyphil, Hyphob letters
    assert head[1] == "%.15g" % st["pos"][0, 0]
    got, t = read_xyz(str(f))
    assert t == 123
    r15 = np.vectorize(lambda v: float("%.15g" % v))
    for k in ("pos", "vel", "acc"):
        assert np.array_equal(got[k], r15(st[k])), k
    assert np.array_equal(got["vel_buf"], got["vel"])
    for k in ("id", "prop", "amp_id", "unit"):
        assert np.array_equal(got[k], st[k]), k
    # appended frames; the reader takes a single frame
    write_xyz(str(f), st, 124, append=True)
    with pytest.raises(EngineError, match="more rows"):
        read_xyz(str(f))


def test_xyz_header_and_capacity_errors(tmp_path):
    f = tmp_path / "init_config.xyz"
    f.write_text("2\nstep 5\n")
    with pytest.raises(EngineError, match="header"):
        read_xyz(str(f))
    st = configs.liquid(np.array([4.0, 4.0, 4.0]), 1.0, seed=2)
    write_xyz(str(f), st, 0)
    with pytest.raises(EngineError, match="CAPACITY"):
        read_xyz(str(f), cap=len(st["pos"]) - 1)


def _bond_lengths(st, box):
    pos = st["pos"].reshape(-1, 4, 3)
    d = np.diff(pos, axis=1)
    d -= box * np.round(d / box)
    return np.linalg.norm(d, axis=2)


def test_sphere_and_cylinder_bilayers():
    box = np.array([30.0, 30.0, 30.0])
    sph = configs.sphere_vesicle(box, 6000, sph_rad=8.0, lip_len=0.5, seed=1)
    assert len(sph["pos"]) == 24000
    assert np.allclose(_bond_lengths(sph, box), configs.BOND_LENG)
    # heads of the outer leaflet point away from the centre
    r = np.linalg.norm(sph["pos"] - 0.5 * box, axis=1).reshape(-1, 4)
    outer = r[:, 0] > 8.0  # the outer leaflet fills first, the rest goes inside
    assert outer.any() and (~outer).any()
    assert np.all(r[outer, 0] > r[outer, 3]) and np.all(r[~outer, 0] < r[~outer, 3])
    cyl = configs.cylinder_bilayer(box, 1500, cyl_r=6.0, axis=2, lip_len=0.5, seed=2)
    assert len(cyl["pos"]) == 6000
    assert np.allclose(_bond_lengths(cyl, box), configs.BOND_LENG)
    rho = np.linalg.norm(cyl["pos"][:, :2] - 15.0, axis=1)
    # beads lie within one molecule length of the mid-radius (heads outermost / innermost)
    assert np.all(np.abs(rho - 6.0) <= configs.ALL_UNIT * configs.BOND_LENG + 1e-9)
    with pytest.raises(ValueError):
        configs.sphere_vesicle(box, 100000, sph_rad=8.0)
