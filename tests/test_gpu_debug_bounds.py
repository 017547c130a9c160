"""The bounds-checking debug library (FSPH_DEBUG_BOUNDS=1, built by
``python -m fltk_sph_ice_gb300.build --debug-bounds``).

Every neighbour slot, cell-table row, list count and boundary slot the passes
read is checked before use; a failed check sets a bit of
fsph_step_stats.bounds_bits and fails the step.  On the scenes below no check
may fail, and since the checks change no arithmetic the debug library must
step bit for bit as the product library does.  Both run the same script in a
child process (FSPH_LIBRARY names the library to load)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from fltk_sph_ice_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
from fltk_sph_ice_gb300 import PBFBatch, abi, rxPBDSPH, rxSPH, scenes

out = {}


def run(cls, sc, steps, tag, boundary=None):
    ps = cls(sc.params)
    ps.Set(sc.pos, sc.vel)
    if boundary is not None:
        ps.SetBoundary(boundary)
    bits = 0
    for _ in range(steps):
        ps.Update(sc.dt)
        bits |= ps.LastStats().bounds_bits
    out[tag + "_x"] = ps.GetArrayVBO(abi.RX_POSITION)
    out[tag + "_v"] = ps.GetArrayVBO(abi.RX_VELOCITY)
    out[tag + "_bits"] = np.array(bits)


for graph in (0, 1):
    sc = scenes.pbf_double_dam_break(block=(24, 24, 48))
    sc.params.use_graph = graph
    sc.params.min_iter, sc.params.max_iter = 2, 8
    run(rxPBDSPH, sc, 30, "pbf%d" % graph)        # lists, in-loop grid rebuilds
sc = scenes.pbf_double_dam_break(block=(16, 16, 32))
sc.params.walk_cells = 1
run(rxPBDSPH, sc, 10, "walk")                     # candidates from the cell rows
sc = scenes.wcsph_dam_break(n_side=24)
run(rxSPH, sc, 20, "wcsph")
sc = scenes.pbf_obstacle_drop(n_side=24)
run(rxPBDSPH, sc, 10, "obstacle", boundary=sc.boundary)   # boundary particles

sc = scenes.batched_scenes(count=5, seed=11, n_lo=512, n_hi=3000)
b = PBFBatch([s.params for s in sc], [s.n for s in sc], iterations=4)
b.set_particles(np.concatenate([s.pos for s in sc]), np.concatenate([s.vel for s in sc]))
bits = 0
for _ in range(3):
    b.step(sc[0].dt)
    for k in range(len(sc)):
        bits |= b.scene_stats(k).bounds_bits
out["batch_x"] = b.get(abi.RX_POSITION)
out["batch_bits"] = np.array(bits)
np.savez(sys.argv[1], **out)
"""


def _run(lib_path, out):
    env = dict(os.environ, FSPH_LIBRARY=lib_path, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", SCRIPT, out], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, f"{lib_path}:\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}"
    return np.load(out)


def test_debug_build_checks_pass_and_steps_match_product(gpu, tmp_path):
    product = build.build()
    debug = build.build(debug_bounds=True)
    assert os.path.dirname(debug) != os.path.dirname(product)
    want = _run(product, str(tmp_path / "product.npz"))
    got = _run(debug, str(tmp_path / "debug.npz"))
    assert sorted(want.files) == sorted(got.files)
    for k in got.files:
        if k.endswith("_bits"):
            assert int(got[k]) == 0, f"{k}: index checks failed (bits {int(got[k])})"
            assert int(want[k]) == 0, f"{k}: the product library reported bounds bits"
        else:
            assert np.array_equal(got[k], want[k]), f"{k}: debug and product steps differ"
