"""The warm-start network's BF16 tensor-core kernels against the numpy oracle
(oracle/mlp.py): forward values, the training gradient, and a training run.

Tolerances: against the BF16-emulating oracle (same rounding points, FP64
sums) 5e-3 in max|a-b| / max|b| per parameter block -- what remains is FP32
summation order and the occasional BF16 tie; against exact FP64 the BF16
error is reported and bounded at 5e-2."""
import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

BLOCKS = {"W1": (omlp.O_W1, omlp.O_B1), "b1": (omlp.O_B1, omlp.O_W2), "W2": (omlp.O_W2, omlp.O_B2),
          "b2": (omlp.O_B2, omlp.O_W3), "W3": (omlp.O_W3, omlp.O_B3), "b3": (omlp.O_B3, omlp.O_SCALE)}


def random_problem(n, seed=0):
    from fltk_sph_ice_gb300 import warmstart
    rng = np.random.default_rng(seed)
    ni = omlp.NI
    x = (rng.standard_normal((n, ni)) * rng.uniform(0.1, 3.0, ni) + rng.uniform(-1, 1, ni)).astype(np.float32)
    t = (rng.standard_normal((n, 3)) * 0.02).astype(np.float32)
    blob = warmstart.init_blob(x, t, seed=seed)
    blob[omlp.O_B1:omlp.O_W2] = rng.standard_normal(64) * 0.1
    blob[omlp.O_B2:omlp.O_W3] = rng.standard_normal(64) * 0.1
    blob[omlp.O_B3:omlp.O_SCALE] = rng.standard_normal(3) * 0.1
    return x, t, blob


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


def test_forward_matches_oracle(gpu):
    from fltk_sph_ice_gb300.warmstart import WarmStartNet
    x, t, blob = random_problem(1000 + 37)  # not a multiple of 16: exercises the padded rows
    net = WarmStartNet(blob)
    y = net.forward(x)
    y_bf, _ = omlp.forward(blob, x, bf16_emul=True)
    y_64, _ = omlp.forward(blob, x, bf16_emul=False)
    print("forward: vs bf16 oracle", rel(y, y_bf), "vs fp64", rel(y, y_64))
    assert rel(y, y_bf) < 5e-3
    assert rel(y, y_64) < 5e-2


def test_gradient_matches_oracle(gpu):
    from fltk_sph_ice_gb300.warmstart import WarmStartNet
    x, t, blob = random_problem(4096 + 100, seed=1)
    net = WarmStartNet(blob)
    g, loss = net.gradient(x, t)
    g_bf, loss_bf = omlp.gradient(blob, x, t, bf16_emul=True)
    g_64, loss_64 = omlp.gradient(blob, x, t, bf16_emul=False)
    assert abs(loss - loss_bf) <= 5e-3 * loss_bf
    report = {}
    for k, (a, b) in BLOCKS.items():
        report[k] = (rel(g[a:b], g_bf[a:b]), rel(g[a:b], g_64[a:b]))
        assert report[k][0] < 5e-3, (k, report[k])
        assert report[k][1] < 5e-2, (k, report[k])
    assert np.all(g[:omlp.O_W1] == 0) and g[omlp.O_SCALE] == 0
    print("gradient rel err (bf16 oracle, fp64 oracle):", report)


def test_training_reduces_loss(gpu):
    """Regression onto a fixed teacher network: Adam on the GPU kernels."""
    from fltk_sph_ice_gb300 import warmstart
    rng = np.random.default_rng(3)
    x = rng.standard_normal((65536, omlp.NI)).astype(np.float32)
    _, _, teacher = random_problem(16, seed=7)
    teacher[omlp.O_MU:omlp.O_SIG] = 0.0
    teacher[omlp.O_SIG:omlp.O_W1] = 1.0
    t, _ = omlp.forward(teacher, x)
    t = t.astype(np.float32)
    blob = warmstart.init_blob(x, t, seed=11)
    net = warmstart.WarmStartNet(blob)
    _, loss0 = net.gradient(x[:8192], t[:8192])
    hist = net.train(x, t, epochs=16, batch=4096, lr=3e-3)
    _, loss1 = net.gradient(x[:8192], t[:8192])
    print("loss", loss0, "->", loss1, hist)
    assert loss1 < 0.1 * loss0
    assert all(np.isfinite(hist))
