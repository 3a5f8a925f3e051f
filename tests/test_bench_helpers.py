"""bench.py's host-side helpers on the CPU: the committed ncu summaries it reads
its roofline traffic and FP64 instruction counts from (every kernel and
precision of the default workload must have one), the launch count it claims,
the healthy-range caps of the late window and the end-to-end solve, and the
variant tags that key the profile tables."""
import argparse

import pytest

import bench


def args(**kw):
    a = argparse.Namespace(workload="taylor_bar", algorithm="usl", basis="linear", material="j2", precision="f64",
                           steps=40, sort_interval=0, alpha=1.0)
    for k, v in kw.items():
        setattr(a, k, v)
    return a


@pytest.mark.parametrize("kernel", ["p2g", "g2p"])
@pytest.mark.parametrize("precision", ["f64", "f32", "dw"])
def test_committed_traffic_for_the_default_workload(kernel, precision):
    t = bench.ncu_traffic(kernel, precision)
    assert t is not None, f"profiles/{kernel}_taylor_bar_{precision}.txt lacks its traffic line"
    # DRAM bytes per launch of 511,784 particles: between the hat-cache-free minimum
    # and twice the algorithmic bytes
    per = t / 511784
    alg = bench.BYTES[precision][kernel]
    assert 0.2 * alg < per < 2.0 * alg, (kernel, precision, per, alg)


def test_variant_tables():
    assert bench.ncu_fp64_inst("g2p", "") == pytest.approx(227, abs=1)
    for tag, kern in (("_quad", "g2p"), ("_cubic", "p2g"), ("_musl", "g2p"), ("_jc", "g2p")):
        assert bench.ncu_traffic(kern, "f64", tag) is not None, (tag, kern)
        assert bench.ncu_fp64_inst(kern, tag) > 100
    assert bench.variant_tag(args(basis="quad", material="jc")) == "_quad_jc"
    assert bench.variant_tag(args()) == ""


def test_launch_count():
    # USL, one body: clear + P2G + grid + G2P per step
    assert bench.launches_per_run(args(), 1) == 40 * 4
    assert bench.launches_per_run(args(), 3) == 40 * 8
    assert bench.launches_per_run(args(sort_interval=4), 1) == 40 * 4 + 10 * 5
    assert bench.launches_per_run(args(), 1, p2g="fused") == 1
    assert bench.launches_per_run(args(algorithm="musl"), 1) == 40 * 7


def test_healthy_ranges():
    assert bench.healthy_steps(args()) == bench.healthy_steps(args(precision="dw")) == 1450
    assert bench.healthy_steps(args(precision="f32")) < bench.healthy_steps(args())
    assert bench.BYTES["dw"] == bench.BYTES["f64"]
