"""The warm-start network's inference on the tcgen05 tensor cores
(fsph_mlp_forward_tcgen05; operands in shared memory, FP32 accumulators in
tensor memory) against the numpy oracle and the mma.sync kernel, and a
warm-started step with it (params.mlp_tcgen05 = 1).

Bars as for the mma.sync kernel (tests/test_gpu_mlp.py): 5e-3 in
max|a-b| / max|b| against the BF16-emulating oracle; the two GPU kernels
round at the same points and differ only in FP32 summation order, 1e-3."""
import numpy as np
import pytest

from oracle import mlp as omlp
from test_gpu_mlp import random_problem, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [37, 128, 1000 + 37, 65536 + 5])
def test_tcgen05_forward_matches_oracle_and_mma_sync(gpu, n):
    from fltk_sph_ice_gb300.warmstart import WarmStartNet
    x, _, blob = random_problem(n, seed=n)
    net = WarmStartNet(blob)
    y_tc = net.forward(x, tcgen05=True)
    y_mma = net.forward(x)
    y_bf, _ = omlp.forward(blob, x, bf16_emul=True)
    print(f"n {n}: tcgen05 vs bf16 oracle {rel(y_tc, y_bf):.2e}, vs mma.sync {rel(y_tc, y_mma):.2e}")
    assert np.isfinite(y_tc).all()
    assert rel(y_tc, y_bf) < 5e-3
    assert rel(y_tc, y_mma) < 1e-3
    # a second call gives the same values (no state carried between calls)
    assert np.array_equal(net.forward(x, tcgen05=True), y_tc)


def test_tcgen05_warm_start_step(gpu):
    """20 warm-started steps of a double dam break with each inference kernel:
    the same iteration counts within one per step.  Positions are compared
    after 3 steps: later, a step that stops one iteration earlier or later
    (both within the tolerance) sends the two runs apart the way any two
    converged solves of this flow part."""
    from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes, warmstart
    blob, _ = warmstart.load_model()
    sc = scenes.pbf_double_dam_break(block=(24, 24, 48))
    out = {}
    for tc in (0, 1):
        p = abi.FsphParams.from_buffer_copy(sc.params)
        p.warm_start, p.mlp_tcgen05 = 1, tc
        p.eta, p.error_mode, p.clamp_constraint, p.max_iter = 1e-3, abi.ERR_ONE_SIDED, 1, 100
        ps = rxPBDSPH(p)
        ps.SetWarmStartModel(blob)
        ps.Set(sc.pos, sc.vel)
        its = []
        for k in range(20):
            ps.Update(sc.dt)
            its.append(ps.LastStats().iterations)
            assert ps.LastStats().status == abi.OK
            if k == 2:
                x3 = ps.GetArrayVBO(abi.RX_POSITION)[:, :3].astype(np.float64)
        out[tc] = (np.array(its), x3)
    assert np.abs(out[0][0] - out[1][0]).max() <= 1, (out[0][0], out[1][0])
    assert abs(out[0][0].mean() - out[1][0].mean()) <= 0.5
    assert np.abs(out[0][1] - out[1][1]).max() < 1e-3 * sc.params.h


@pytest.mark.parametrize("n", [5, 100, 4096, 1 << 20])
def test_tma_inputs_step_identically(gpu, n):
    """The committed network weights only the 16 local inputs; with
    mlp_tcgen05 = 1 their rows reach shared memory as TMA boxes
    (cp.async.bulk.tensor, rows past n filled with zeros), with 2 by
    per-thread loads.  Same arithmetic after that, so the warm-started
    steps are bit-identical, including a last, partial 128-row tile."""
    from fltk_sph_ice_gb300 import abi, rxPBDSPH, scenes, warmstart
    blob, _ = warmstart.load_model()
    side = 64 if n == 1 << 20 else 8
    sc = scenes.pbf_double_dam_break(block=(side, side, 2 * side))
    keep = sc.n - 37 if n >= 4096 else n  # a partial last tile; fewer rows than one tile
    out = []
    for mode in (1, 2):
        p = abi.FsphParams.from_buffer_copy(sc.params)
        p.warm_start, p.mlp_tcgen05 = 1, mode
        p.max_iter = 60
        ps = rxPBDSPH(p)
        ps.SetWarmStartModel(blob)
        ps.Set(sc.pos[:keep], sc.vel[:keep])
        its = []
        for _ in range(4):
            ps.Update(sc.dt)
            its.append(ps.LastStats().iterations)
            assert ps.LastStats().status in (abi.OK, abi.NOT_CONVERGED)
        out.append((its, ps.GetArrayVBO(abi.RX_POSITION), ps.GetArrayVBO(abi.RX_STEP_CORRECTION)))
        ps.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
    if keep > 100:
        assert np.abs(out[0][2][:, :3]).max() > 0  # the network ran
