"""The committed warm-start network and the training options, on the CPU:
blob layout, the unweighted-input convention (an input whose sigma is at
least 1e29 carries no weight) and the oracle network's response to it."""
import json
import os

import numpy as np

import oracle.mlp as omlp
from fltk_sph_ice_gb300 import abi, warmstart


def _committed():
    assert os.path.isfile(warmstart.DEFAULT_MODEL)
    return warmstart.load_model(warmstart.DEFAULT_MODEL)


def test_committed_blob_layout():
    blob, meta = _committed()
    assert blob.shape == (abi.MLP_BLOB_SIZE,) == (omlp.BLOB,)
    assert np.isfinite(blob).all()
    assert blob[warmstart.O_SCALE] > 0
    assert meta["epochs"] > 0 and len(meta["loss"]) == meta["epochs"]
    assert 0.5 <= meta["output_damping"] <= 1.0


def test_committed_network_weights_only_what_its_record_says():
    blob, meta = _committed()
    sig = blob[warmstart.O_SIG:warmstart.O_W1]
    local = sig[:warmstart.BASE_FEATURES]
    assert (local < 1e29).all()
    if meta.get("features") == "base":
        assert (sig[warmstart.BASE_FEATURES:] >= 1e29).all()


def test_unweighted_inputs_do_not_change_the_output():
    """With sigma >= 1e29 on inputs 16-31, any finite values there leave the
    network's output unchanged (FP64 oracle, and with the BF16 rounding the
    kernels apply)."""
    blob, _ = _committed()
    b = np.array(blob, np.float32)
    b[warmstart.O_SIG + warmstart.BASE_FEATURES:warmstart.O_W1] = np.float32(1e30)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((257, abi.MLP_FEATURES)).astype(np.float32)
    x2 = x.copy()
    x2[:, warmstart.BASE_FEATURES:] = rng.uniform(-1e3, 1e3, (257, abi.MLP_FEATURES - warmstart.BASE_FEATURES))
    for emul in (False, True):
        y1, _ = omlp.forward(b, x, bf16_emul=emul)
        y2, _ = omlp.forward(b, x2, bf16_emul=emul)
        assert np.allclose(y1, y2, rtol=0, atol=1e-12 * max(1.0, np.abs(y1).max()))


def test_training_record_is_json():
    _, meta = _committed()
    json.dumps(meta)
    for k in ("samples", "rollouts", "epochs", "loss", "damping_table"):
        assert k in meta


def test_training_scene_sizes():
    """The stated particle ranges of the three training distributions
    (4 bx^2 by particles per double dam break)."""
    for sizes, lo, hi, tall in (("config", 65536, 262144, 1.0), ("large", 65536, 262144, 2.0),
                                ("small", 16000, 131072, 1.0)):
        rng = np.random.default_rng(12345)
        for _ in range(500):
            bx, by, bz = warmstart.next_block(sizes, rng)
            n = 4 * bx * bx * by
            assert bz == 2 * bx and lo <= n <= hi, (sizes, bx, by, n)
            assert by <= tall * bx


def test_seed_selection():
    assert warmstart.select_seed({0: 5.65, 1: 4.86, 2: 6.95, 4: 4.33, 5: 4.94}) == 4
    assert warmstart.select_seed({3: 2.0, 1: 2.0}) == 1


def test_damping_calibration_picks_fewest_iterations(monkeypatch):
    """calibrate_damping scores every alpha on the held-out scenes and keeps
    the one with the fewest mean iterations (solver calls replaced by a fake)."""
    blob, _ = _committed()
    seen = []

    def fake(b, block, seed, steps=60, skip=30):
        a = float(b[warmstart.O_SCALE] / blob[warmstart.O_SCALE])
        seen.append((round(a, 3), seed))
        return 10.0 + 40.0 * (a - 0.8) ** 2 + seed * 1e-3

    monkeypatch.setattr(warmstart, "mean_iterations", fake)
    alpha, table = warmstart.calibrate_damping(blob)
    assert alpha == 0.8
    assert sorted(table) == [0.6, 0.7, 0.8, 0.9, 1.0]
    assert len(seen) == 5 * len(warmstart.CALIB_SCENES)
    assert {s for _, s in seen} == {s for _, s in warmstart.CALIB_SCENES}


def test_validation_score_is_the_mean_over_the_validation_scenes(monkeypatch):
    calls = []

    def fake(b, block, seed, steps=60, skip=30):
        calls.append((block, seed, steps, skip))
        return float(seed - 590)

    monkeypatch.setattr(warmstart, "mean_iterations", fake)
    v = warmstart.validation_iterations(np.zeros(abi.MLP_BLOB_SIZE, np.float32))
    assert [c[:2] for c in calls] == [tuple(s) for s in warmstart.VALID_SCENES]
    assert all(c[2] == 144 and c[3] == 104 for c in calls)
    assert v == np.mean([s - 590 for _, s in warmstart.VALID_SCENES])
    # validation scenes are neither calibration nor training scenes
    assert not {s for _, s in warmstart.VALID_SCENES} & {s for _, s in warmstart.CALIB_SCENES}
    assert all(s < 1000 for _, s in warmstart.VALID_SCENES)
