"""The bounds-checked build (every gather of the matched and batched kernels
verifies its index and counts violations) runs every kernel form over a set
of geometries -- mirrored and general cone, helix, odd sizes, short source
distance, both fan block shapes, batches, fused CGLS -- without a single
out-of-range index."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_no_gather_leaves_its_array():
    from framelab_gb300 import build as B
    B.build(variant="checked")
    env = dict(os.environ, FRAMELAB_GB300_VARIANT="checked")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "gpu_bounds_script.py")],
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("violations")][-1]
    assert int(line.split()[1]) == 0, line
