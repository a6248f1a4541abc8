"""CPU legs of bench.py that need no GPU: the single-core baseline of the
headline line, and the mixed-size stream labelled by the reference's CPU path
on every host core (spawned processes reading the volumes from one
memory-mapped file), which must label every volume."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(300)
def test_stream_on_all_cores():
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    from cc3d_gb300 import synth
    oracle.build()
    shapes = synth.batch_shapes(24, 8, 40, seed=3)
    vols = [synth.voronoi_volume(s, max(1, int(np.prod(s)) // 512), 65535, seed=i, dtype=np.uint16, salt=0.0)
            for i, s in enumerate(shapes)]
    res = bench.cpu_stream_all_cores(vols, "port", reps=1)
    assert res["cores"] >= 1 and res["kind"] == "port" and res["value"] > 0
    assert f"({sum(v.size for v in vols)} voxels)" in res["sample"]


def test_single_core_baseline():
    """The GPU arm's CPU baseline: the reference's CPU path on one core, best of
    up to three runs, with the host's CPU model."""
    sys.path.insert(0, ROOT)
    import bench
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((40, 48, 56), 24, 1 << 20, seed=3)
    res = bench.cpu_reference(vol, budget_s=5.0)
    assert res["cores"] == 1 and res["value"] > 0 and res["cpu_model"]
    assert res["kind"] in ("reference", "port")
