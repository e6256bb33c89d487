"""The bench's roofline bookkeeping on the CPU: which single-kernel phase it
reports, the algorithmic bytes it divides by, and the committed ncu
summaries it reads the measured traffic from."""
import json
import os

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _phases(**ms):
    return [ms.get(p, 0.0) for p in bench.PHASES]


def test_phase_list_times_the_particle_triangle_law_apart_from_its_probe():
    assert len(bench.PHASES) == 9
    assert bench.PHASES.index("pt_items") + 1 == bench.PHASES.index("pt_law")


def test_the_longest_single_kernel_phase_is_reported():
    n, sides, hv, L = 2_000_000, 3_800_000, 48, 2.0
    name, kernel, ms, nbytes = bench.dominant_kernel(_phases(sweep=0.27, pp_law=0.18, owner_sum=0.08, pt_items=0.5,
                                                             pt_law=0.22), n, sides, hv, L, items=20_000,
                                                     manifolds=17_000)
    # the item probe is not a candidate even when it is the longest phase
    assert (name, kernel, ms) == ("sweep", "k_sweep", 0.27)
    assert nbytes == pytest.approx(n * (116 + 4 + 8 * L) + sides * 28)


@pytest.mark.parametrize("items,kernel", [(20_000, "k_pt_thread"), (200, "k_pt_warp")])
def test_the_particle_triangle_law_is_reported_with_its_own_bytes(items, kernel):
    name, k, ms, nbytes = bench.dominant_kernel(_phases(sweep=0.04, pp_law=0.03, pt_law=0.07), 200_000, 388_000, 48,
                                                2.0, items=items, manifolds=143)
    assert (name, k, ms) == ("pt_law", kernel, 0.07)
    assert nbytes == bench.pt_bytes(items, 143, 108)


def test_no_items_no_particle_triangle_candidate():
    name, _, _, _ = bench.dominant_kernel(_phases(sweep=0.01, pt_law=0.5), 1000, 2000, 48, 2.0, items=0)
    assert name == "sweep"


def test_fp64_figures_come_from_the_committed_captures():
    out = bench.fp64_roofline(_phases(pt_law=0.2, pp_law=2.9), "c2", "fp64")
    assert set(out) == {"k_pp_law<double>", "k_pt_thread"}
    assert out["k_pt_thread"]["phase_ms"] == 0.2
    assert 0.0 < out["k_pt_thread"]["fp64_pipe_active_frac"] <= 1.0
    out1 = bench.fp64_roofline(_phases(pt_law=0.07), "c1", "mixed")
    assert set(out1) == {"k_pt_warp"}


def test_every_traffic_record_names_a_committed_summary():
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        records = json.load(f)
    for config, kernels in records.items():
        for kernel, rec in kernels.items():
            assert os.path.exists(os.path.join(ROOT, rec["source"])), (config, kernel)
            assert rec["bytes_per_particle"] > 0 and rec["particles"] > 0
