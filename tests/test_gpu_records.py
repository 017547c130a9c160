"""The step record and the allocation-failure paths on the GPU.

The per-step JSON-lines log carries what the reference kept in its globals
g_iIterations / g_fEta (rx_sph_pbd.cpp:461-462).  Allocation failures are
injected on the host (fsph_set_alloc_fault refuses the allocation before
cudaMalloc is called), so no device fault is involved: every refused
allocation must come back as FSPH_OOM, leak nothing, and leave a context
that refuses work until fsph_set_params reallocates it."""
import json

import numpy as np
import pytest

from fltk_sph_ice_gb300 import FsphError, abi, rxPBDSPH, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture
def no_faults():
    abi.set_alloc_fault(-1, -1)
    yield
    abi.set_alloc_fault(-1, -1)


def _scene():
    sc = scenes.pbf_double_dam_break(block=(10, 10, 20))
    p = sc.params
    p.max_iter, p.min_iter = 6, 2
    return sc, p


def test_step_log_lines(gpu, tmp_path):
    sc, p = _scene()
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    log = tmp_path / "steps.jsonl"
    ps.SetStepLog(str(log))
    stats = []
    for _ in range(3):
        ps.Update(sc.dt)
        s = ps.LastStats()
        stats.append((s.iterations, s.density_error))
    ps.SetStepLog(None)
    ps.Update(sc.dt)  # not logged
    rec = [json.loads(line) for line in log.read_text().splitlines()]
    assert [r["step"] for r in rec] == [0, 1, 2]
    for r, (it, err) in zip(rec, stats):
        assert r["solver"] == "pbf" and r["n"] == sc.n == r["n_active"]
        assert r["iterations"] == it and p.min_iter <= it <= p.max_iter
        assert r["density_error"] == pytest.approx(err, rel=1e-6)
        assert r["status"] in ("FSPH_OK", "FSPH_NOT_CONVERGED") and r["host_ms"] > 0.0
        assert abs(r["dt"] - sc.dt) < 1e-9


def test_every_refused_create_allocation_is_reported_and_freed(gpu, no_faults):
    torch = pytest.importorskip("torch")
    sc, p = _scene()
    rxPBDSPH(p).close()  # warm the allocator and the module
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    refused = 0
    for k in range(80):
        abi.set_alloc_fault(-1, k)
        try:
            ps = rxPBDSPH(p)
        except FsphError as e:
            assert e.status == abi.OOM
            refused += 1
            continue
        ps.close()
        break
    else:
        pytest.fail("create still refused after 80 allocations")
    assert refused >= 20  # the particle, list and grid buffers
    torch.cuda.synchronize()
    assert free0 - torch.cuda.mem_get_info()[0] < (16 << 20)


def test_size_cap_refuses_large_contexts(gpu, no_faults):
    sc, p = _scene()
    abi.set_alloc_fault(4 << 20, -1)
    big = abi.FsphParams.from_buffer_copy(p)
    big.max_particles = 1 << 20  # 16 MiB position arrays
    with pytest.raises(FsphError) as e:
        rxPBDSPH(big)
    assert e.value.status == abi.OOM
    ps = rxPBDSPH(p)  # the small one fits under the cap
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)


def test_failed_reallocation_leaves_a_refusing_context(gpu, no_faults):
    sc, p = _scene()
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)
    bigger = abi.FsphParams.from_buffer_copy(p)
    bigger.max_particles = p.max_particles * 2
    abi.set_alloc_fault(-1, 3)  # part-way through the new particle buffers
    with pytest.raises(FsphError) as e:
        ps.SetParams(bigger)
    assert e.value.status == abi.OOM
    abi.set_alloc_fault(-1, -1)
    for call in (lambda: ps.Update(sc.dt), lambda: ps.GetArrayVBO(abi.RX_POSITION), lambda: ps.Set(sc.pos, sc.vel),
                 lambda: ps.SetParticlesToCell()):
        with pytest.raises(FsphError) as e:
            call()
        assert e.value.status == abi.OOM
    ps.SetParams(bigger)  # reallocates everything; the particles were lost
    assert ps.GetNumParticles() == 0 and ps.GetMaxParticles() == bigger.max_particles
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)
    x = ps.GetArrayVBO(abi.RX_POSITION)
    assert x.shape[0] == sc.n and np.isfinite(x).all()


def test_failed_grid_reallocation_keeps_refusing_until_reset(gpu, no_faults):
    sc, p = _scene()
    ps = rxPBDSPH(p)
    ps.Set(sc.pos, sc.vel)
    wider = abi.FsphParams.from_buffer_copy(p)
    wider.box_max[0] = p.box_max[0] + 0.5  # more cells: the grid is reallocated
    abi.set_alloc_fault(-1, 1)
    with pytest.raises(FsphError):
        ps.SetParams(wider)
    abi.set_alloc_fault(-1, -1)
    with pytest.raises(FsphError):
        ps.Update(sc.dt)
    ps.SetParams(wider)
    ps.Set(sc.pos, sc.vel)
    ps.Update(sc.dt)
    assert np.isfinite(ps.GetArrayVBO(abi.RX_POSITION)).all()
