"""Asynchronous trajectory frames (idpd_dump_xyz_async): frames queued while
the steps go on must be byte-identical to frames written from synchronous
downloads of the same steps (idpd_download_state + idpd_write_xyz), in the
reference's traject.xyz format, across storage reorders."""
import os

import pytest

from helpers import mdpd_params, mixed_system
from implicit_dpd_gb300.engine import Engine, EngineError, write_xyz

pytestmark = pytest.mark.gpu


def _run(box, st, n_amp, p, tmp, async_frames):
    e = Engine(sort_period=7)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp)
    e.set_tuning(1, 0.2)
    path = os.path.join(tmp, "async.xyz" if async_frames else "sync.xyz")
    for k in range(4):
        e.step(9)  # crosses storage reorders (every 7 steps)
        if async_frames:
            e.dump_xyz_async(path, append=k > 0)
        else:
            s = e.download()
            write_xyz(path, s, e.get_params().time, append=k > 0)
    if async_frames:
        e.dump_wait()
    e.close()
    return open(path, "rb").read()


def test_async_frames_equal_synchronous_frames(tmp_path):
    box, st, n_amp = mixed_system(seed=17)
    p = mdpd_params(box, time=3)
    a = _run(box, st, n_amp, p, str(tmp_path), True)
    b = _run(box, st, n_amp, p, str(tmp_path), False)
    assert a == b
    assert a.count(b"time ") == 4


def test_async_frame_write_error_is_reported(tmp_path):
    box, st, n_amp = mixed_system(seed=1)
    e = Engine()
    e.set_params(mdpd_params(box))
    e.upload(st)
    e.step(1)
    e.dump_xyz_async(str(tmp_path / "no_such_dir" / "x.xyz"), append=False)
    with pytest.raises(EngineError, match="cannot open"):
        e.dump_wait()
    e.dump_wait()  # the error is reported once
    e.close()
