"""StateRecorder output of a GPU run against the reference's own files for the same run (golden
fixture tests/golden/recorder.npz: the raw bytes the reference's StateRecorder wrote with
collectDiagnostics and recordField).

Same file set and sizes, identical binary headers (particle count, frame count); frames: positions
within 2e-6 of the box scale, fields (original-unit accelerations) within 3e-5 RMS relative;
text: same line counts, energies within 2e-6 (the reference prints 6 decimals), vectors within
1e-5 of their largest component (the reference prints %.6e of float sums).
"""
import os
import struct

import numpy as np
import pytest

from conftest import load_npz, rel_rms
from test_gpu_pm import make_pm
from test_oracle_pin import cfg_from

pytestmark = pytest.mark.gpu

REC = load_npz("recorder.npz")


def frames_of(b):
    n, frames = struct.unpack("<ii", b[:8])
    data = np.frombuffer(b[8:], np.float32).reshape(-1, n, 3)
    return (n, frames), data


def text_of(b):
    lines = [l for l in b.decode().splitlines() if l.strip()]
    return np.array([[float(x) for x in l.split()] for l in lines]).reshape(len(lines), -1)


@pytest.mark.parametrize("case", ["ext", "escape"])
def test_recorder_files_match_reference(gpu_lib, case, tmp_path):
    import particlesimulation_gb300 as P
    d = REC[case]
    ref = {k[len("file:"):]: d[k].tobytes() for k in d if k.startswith("file:")}
    cfg = cfg_from(d)
    n, steps = len(d["mass"]), int(d["sim_length"])
    pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    rec = P.StateRecorder(n, steps + 1, tmp_path)
    esc, _ = pm.run(steps, collectDiagnostics=True, stateRecorder=rec, recordField=True)
    assert esc == bool(d["escaped"])
    assert rec.flush() == str(tmp_path)
    ours = {}
    for name in sorted(os.listdir(tmp_path)):
        with open(os.path.join(tmp_path, name), "rb") as f:
            ours[name] = f.read()
    assert sorted(ours) == sorted(ref)
    for name in ("positions.dat", "field.dat"):
        assert len(ours[name]) == len(ref[name]), name
        (h1, a), (h2, b) = frames_of(ours[name]), frames_of(ref[name])
        assert h1 == h2 == (n, steps + 1)
        if name == "positions.dat":
            assert np.abs(a - b).max() < 2e-6 * np.abs(b).max()
        else:
            for k in range(len(a)):
                assert rel_rms(a[k], b[k]) < 3e-5, (name, k)
    for name in ("energy.txt", "momentum.txt", "expected_momentum.txt", "angular_momentum.txt"):
        a, b = text_of(ours[name]), text_of(ref[name])
        assert a.shape == b.shape, name
        if name == "energy.txt":
            assert np.abs(a - b).max() < 2e-6
        else:
            assert np.abs(a - b).max() < 1e-5 * np.abs(b).max(), name
    assert rec.framesWritten() == len(frames_of(ours["positions.dat"])[1])
    rec.close()
    pm.close()


def test_recorder_many_frames_and_empty_names(gpu_lib, tmp_path):
    """More frames than one device buffer holds (the frames cross buffer swaps in order), and
    outputs left out by empty names, as the reference's demos do."""
    import particlesimulation_gb300 as P
    d = REC["ext"]
    cfg = cfg_from(d)
    n = len(d["mass"])
    pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    steps = 150
    rec = P.StateRecorder(n, steps + 1, tmp_path, "pos.dat", "", "", "", "", "", withField=False)
    esc, done = pm.run(steps, stateRecorder=rec)
    assert not esc and done == steps + 1
    assert sorted(os.listdir(tmp_path)) == ["pos.dat"]
    with open(os.path.join(tmp_path, "pos.dat"), "rb") as f:
        hdr, frames = frames_of(f.read())
    assert hdr == (n, steps + 1) and len(frames) == steps + 1
    # the last frame is the final state, the first one the state after the first drift
    x, _, _ = pm.getParticles(units="original")
    assert np.abs(frames[-1] - x).max() < 1e-5 * np.abs(x).max()
    assert not np.array_equal(frames[0], frames[1])
    rec.close()
    pm.close()
