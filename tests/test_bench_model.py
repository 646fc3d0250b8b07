"""The bench's accounting, without a GPU: the algorithmic bytes per cell and
RK stage of each path (the roofline's numerator) and the choice of the probe
ring reported for the acoustic error."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

STEP_KERNELS = ("k_prep", "k_grad", "k_vis", "k_flux", "k_update")


def _step(dim, fpc, fp32, scheme, viscous):
    kb = bench.kernel_bytes(dim, fpc, fp32, scheme, viscous)
    return sum(kb[k] for k in STEP_KERNELS)


@pytest.mark.parametrize("dim,fpc,fp32,scheme,viscous,expected", [
    (2, 4, False, "M1", True, 738.0),    # the headline: 768x512 cylinder, FP64
    (2, 4, True, "M1", True, 442.0),     # the same, FP32-bulk
    (3, 6, True, "M2", True, 703.0),     # the 9.4M-cell wake, FP32-bulk
    (3, 6, False, "M2", True, 1203.0),   # the wake, FP64
])
def test_step_bytes_per_cell(dim, fpc, fp32, scheme, viscous, expected):
    assert _step(dim, fpc, fp32, scheme, viscous) == pytest.approx(expected)


def test_fused_kernels_do_the_separate_kernels_work():
    """The fused flux + update touches the two kernels' bytes less the face
    rhs it never stores or reads back; the tile stage, every kernel's."""
    kb = bench.kernel_bytes(2, 4, True, "M1", False)
    assert kb["k_flux_update"] == pytest.approx(kb["k_flux"] + kb["k_update"] - 2 * 2 * 4 * 4)
    assert kb["k_tile_stage"] == pytest.approx(sum(kb[k] for k in ("k_grad", "k_vis", "k_flux", "k_update")))


def _ck(steps, rel):
    return {"steps": steps, "probe_rings": [{"radius": 5.0, "rel_l2": 1e-6, "p_rms_ref": 10.0},
                                            {"radius": 50.0, "rel_l2": rel, "p_rms_ref": 0.0 if rel is None else 5.0}]}


def test_probe_ring_taken_where_the_pulse_has_arrived():
    ring = bench.ring_at_longest([_ck(20000, None), _ck(80000, 9.7e-7)], 50.0)
    assert ring["steps"] == 80000 and ring["rel_l2"] == 9.7e-7
    ring = bench.ring_at_longest([_ck(20000, 3e-7), _ck(80000, 9.7e-7)], 50.0)
    assert ring["steps"] == 80000
    ring = bench.ring_at_longest([_ck(20000, 3e-7), _ck(80000, None)], 50.0)
    assert ring["steps"] == 20000 and ring["rel_l2"] == 3e-7
    ring = bench.ring_at_longest([_ck(20000, None)], 50.0)
    assert ring["steps"] == 20000 and ring["rel_l2"] is None
