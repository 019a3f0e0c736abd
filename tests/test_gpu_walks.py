"""The FDPS multi-walk interface (DispatchKernel / RetrieveKernel of the
reference's GPU hook, f_calculator_gpu.cuh:9-21) against the oracle.

Walks are built the way FDPS's short-range tree builds them: the i particles
of one cell of side >= 1.2 (the search radius) and, as j particles, every
particle of the 27 surrounding cells with its periodic image shift applied.
The records use the reference's EPI / EPJ / RESULT layouts.
"""
import numpy as np
import pytest

import pyoracle as O
from helpers import FORCE_TOL, mdpd_params, mixed_system, rel_force_err
from implicit_dpd_gb300.abi import WALK_DENSITY, WALK_FORCE
from implicit_dpd_gb300.engine import WALK_DTYPES, Engine

pytestmark = pytest.mark.gpu


def _walks(pos, box):
    nc, cell_of, start, members = O.cells(pos, box, 1.2)
    nc = np.asarray(nc)
    walks = []
    for c in range(int(np.prod(nc))):
        ii = members[start[c]:start[c + 1]]
        if len(ii) == 0:
            continue
        cx, cy, cz = c % nc[0], (c // nc[0]) % nc[1], c // (nc[0] * nc[1])
        js, shifts = [], []
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    q = np.array([cx + dx, cy + dy, cz + dz])
                    s = np.floor_divide(q, nc)
                    w = q - s * nc
                    cn = w[0] + nc[0] * (w[1] + nc[1] * w[2])
                    jj = members[start[cn]:start[cn + 1]]
                    js.append(jj)
                    shifts.append(np.repeat((s * box)[None, :], len(jj), axis=0))
        walks.append((ii, np.concatenate(js), np.concatenate(shifts)))
    return walks


def test_walk_density_and_force_match_oracle():
    box, st, _ = mixed_system()
    p = mdpd_params(box, time=31)
    dens, cm, cnt = O.density(p, st["pos"], st["prop"], nthreads=4)
    acc, press = O.force(p, st["pos"], st["vel"], st["id"], st["prop"], dens, nthreads=4)
    walks = _walks(st["pos"], box)
    e = Engine()
    e.set_params(p)
    ti, tj, _ = WALK_DTYPES[WALK_DENSITY]
    epi, epj = [], []
    for ii, jj, sh in walks:
        a = np.zeros(len(ii), ti)
        a["prop"], a["pos"] = st["prop"][ii], st["pos"][ii]
        b = np.zeros(len(jj), tj)
        b["prop"], b["pos"] = st["prop"][jj], st["pos"][jj] + sh
        epi.append(a)
        epj.append(b)
    e.dispatch_walks(WALK_DENSITY, epi, epj, tag=7)
    res = e.retrieve_walks(WALK_DENSITY, tag=7)
    got_d = np.zeros_like(dens)
    got_cm = np.zeros((len(dens), 6))
    got_cnt = np.zeros((len(dens), 2), np.uint32)
    for (ii, _, _), r in zip(walks, res):
        got_d[ii] = r["dens"]
        got_cnt[ii] = r["nei_cnt"]
        with np.errstate(invalid="ignore", divide="ignore"):
            got_cm[ii, :3] = r["nei_pos_sum"][:, 0] / r["nei_cnt"][:, 0:1]
            got_cm[ii, 3:] = r["nei_pos_sum"][:, 1] / r["nei_cnt"][:, 1:2]
    assert np.abs(got_d - dens).max() / np.abs(dens).max() < FORCE_TOL
    assert np.array_equal(got_cnt, np.asarray(cnt, np.uint32))
    ok = np.isfinite(cm)
    assert np.array_equal(np.isfinite(got_cm), ok)
    assert np.abs(got_cm[ok] - cm[ok]).max() < 1e-12

    ti, tj, _ = WALK_DTYPES[WALK_FORCE]
    epi, epj = [], []
    for ii, jj, sh in walks:
        a = np.zeros(len(ii), ti)
        a["id"], a["prop"], a["pos"], a["vel"], a["dens"] = (st["id"][ii], st["prop"][ii],
                                                             st["pos"][ii], st["vel"][ii], dens[ii])
        b = np.zeros(len(jj), tj)
        b["id"], b["prop"], b["pos"], b["vel"], b["dens"] = (st["id"][jj], st["prop"][jj],
                                                             st["pos"][jj] + sh, st["vel"][jj],
                                                             dens[jj])
        b["amp_id"], b["unit"] = st["amp_id"][jj], st["unit"][jj]
        epi.append(a)
        epj.append(b)
    e.dispatch_walks(WALK_FORCE, epi, epj, tag=8)
    res = e.retrieve_walks(WALK_FORCE, tag=8)
    got_a = np.zeros_like(acc)
    got_p = np.zeros_like(press)
    for (ii, _, _), r in zip(walks, res):
        got_a[ii] = r["acc"]
        got_p[ii] = r["press"]
    assert rel_force_err(got_a, acc)[0] < FORCE_TOL
    assert np.abs(got_p - press).max() / np.abs(press).max() < 1e-4


def test_walk_retrieve_needs_matching_dispatch():
    box, st, _ = mixed_system()
    e = Engine()
    e.set_params(mdpd_params(box))
    ti, tj, _ = WALK_DTYPES[WALK_DENSITY]
    a = np.zeros(3, ti)
    a["pos"] = st["pos"][:3]
    e.dispatch_walks(WALK_DENSITY, [a], [a.astype(tj)], tag=1)
    from implicit_dpd_gb300.engine import EngineError
    with pytest.raises(EngineError, match="STATE"):
        e.retrieve_walks(WALK_DENSITY, tag=2)
    r = e.retrieve_walks(WALK_DENSITY, tag=1)
    assert r[0]["nei_cnt"][:, 0].min() >= 1  # the particle itself
