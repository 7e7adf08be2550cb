"""State files (save/load/resume) through the C ABI."""
import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHSolver, read_state_file, scene_positions
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def test_save_load_resume_is_bit_exact(tmp_path):
    prm = params_16k(viscosity=0.02)
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    path = str(tmp_path / "state.sfs")
    with SPHSolver(prm) as a:
        a.setParticles(pos)
        a.step(120)
        a.saveState(path, sim_time=0.012)
        saved = a.getState()
        a.step(80)
        ref = a.getState()
    f = read_state_file(path)
    assert f["sim_time"] == 0.012 and f["params"].viscosity == np.float32(0.02)
    assert np.array_equal(f["positions"].view(np.uint32), saved[0].view(np.uint32))
    assert np.array_equal(f["velocities"].view(np.uint32), saved[1].view(np.uint32))
    with SPHSolver(params_16k()) as b:
        t = b.loadState(path)
        assert t == 0.012 and b.params.viscosity == np.float32(0.02)
        b.step(80)
        got = b.getState()
    assert np.array_equal(got[0].view(np.uint32), ref[0].view(np.uint32))
    assert np.array_equal(got[1].view(np.uint32), ref[1].view(np.uint32))


def test_load_rejects_bad_files(tmp_path, lib):
    bad = tmp_path / "bad.sfs"
    bad.write_bytes(b"not a state file")
    with SPHSolver(params_16k()) as s:
        with pytest.raises(C.SFError):
            s.loadState(str(bad))
        with pytest.raises(C.SFError):
            s.loadState(str(tmp_path / "missing.sfs"))
