"""bench.py's host logic (CPU): workload sizes and precision options, and the
serving request stream (seeded, within the configured sizes and path counts,
Poisson arrivals at the configured rate), and the workload the committed ncu
traffic is reported for."""
import sys

import numpy as np


def _bench():
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    return bench


def test_workload_defaults_and_precision_options():
    b = _bench()

    class A:
        workload, dims, size, density, sums, fp64_after = "head_neck", "", 0, "unorm16", "fp32", 0
    a = A()
    assert b.dims_of(a) == "512,512,400" and b.image_size(a) == (1024, 1024)
    a.workload = "torso"
    assert b.dims_of(a) == "512,512,800" and b.image_size(a) == (1920, 1080)
    a.size, a.dims = 256, "64,64,80"
    assert b.image_size(a) == (256, 256) and b.dims_of(a) == "64,64,80"
    a.density, a.sums, a.fp64_after = "bf16", "kahan", 65536
    p = b.precision_of(a)
    assert (p.density_format, p.sums, p.fp64_after) == (2, 1, 65536)
    assert b.precision_of(a, "fp32").density_format == 3


def test_serving_request_stream():
    b = _bench()
    from volview_gb300 import scene
    vols = {"a": scene.torso_config(seed=1, dims=(64, 64, 64), soft=False),
            "b": scene.torso_config(seed=2, dims=(64, 64, 96), soft=False)}
    reqs = b.serve_requests(vols, 400, 40.0, seed=3)
    again = b.serve_requests(vols, 400, 40.0, seed=3)
    assert [(q.volume, q.width, q.height, q.spp, q.arrival) for q in reqs] == \
           [(q.volume, q.width, q.height, q.spp, q.arrival) for q in again]
    assert {(q.width, q.height) for q in reqs} <= set(b.SERVE_SIZES)
    assert {q.spp for q in reqs} <= set(b.SERVE_SPP) and {q.volume for q in reqs} == {"a", "b"}
    gaps = np.diff([0.0] + [q.arrival for q in reqs])
    assert np.all(gaps > 0) and abs(gaps.mean() - 1 / 40.0) < 0.25 / 40.0  # Poisson at 40/s
    hidden = np.mean([[q.params.labels.colors[l][3] == 0.0 for l in range(1, 11)] for q in reqs])
    assert 0.12 < hidden < 0.28  # each label hidden with probability 0.2


def test_ncu_traffic_only_on_the_captured_workload():
    """The DRAM traffic per frame, estimated from ncu captures for the default
    workload: the bench reports it there and nowhere else."""
    b = _bench()

    class A:
        workload, dims, size, density, sums, fp64_after, light_map = "head_neck", "", 0, "unorm16", "fp32", 0, False
    a = A()
    assert b.ncu_traffic(a) is not None and b.ncu_traffic(a) > 0
    for field, value in (("workload", "torso"), ("size", 512), ("dims", "256,256,200"), ("light_map", True),
                         ("density", "bf16")):
        other = A()
        setattr(other, field, value)
        assert b.ncu_traffic(other) is None, field


def test_l2_note_follows_the_volume_sizes():
    b = _bench()

    class A:
        workload, dims, size, density, sums, fp64_after, light_map = "head_neck", "", 0, "unorm16", "fp32", 0, False
    a = A()
    assert b.volume_bytes(a) == 512 * 512 * 400 * 11 and b.l2_note(a).startswith("inputs larger than L2 (1.15 GB")
    a.density = "fp32"
    assert b.volume_bytes(a) == 512 * 512 * 400 * 13
    a.dims = "60,64,80"  # bricked: 64 x 64 x 80
    assert b.volume_bytes(a) == 64 * 64 * 80 * 13 and b.l2_note(a).startswith("inputs smaller than L2")
