"""lfm_solver_residual_noalloc: the entry point that allocates no device memory.

Some callers cannot allocate device memory when they need a residual - code
that runs while a CUDA graph is captured, allocator-free serving loops, or a
host whose device memory belongs to another runtime. This entry point takes
the state and the output as the caller's device buffers and keeps its scratch
in one static device array. The test hands it device buffers owned by the
test (PyTorch tensors), calls it twice in a row on different states, and
compares each result with the residual the regular path records for the same
state (lfm_solver_cell_residual), at the tolerance of the other residual
tests (FP64: 1e-10 relative L2; FP32-bulk: 1e-4 of the largest value per
field; the two paths run the same kernels, so the match is normally exact).
It also hands the state over with a row stride larger than the cell count,
and checks the refusals: a stride below the cell count, a case larger than
the scratch array, and a partition of a decomposed case (whose halo rows the
caller's state does not cover). The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from lfm_public_gb300 import _native as N, cases

pytestmark = pytest.mark.gpu


def _noalloc(s, q_dev, res_dev, stream, stride=None):
    lib = N.load_library()
    rc = lib.lfm_solver_residual_noalloc(s._h, C.c_void_p(q_dev.data_ptr()),
                                         q_dev.shape[1] if stride is None else stride,
                                         C.c_void_p(res_dev.data_ptr()), C.c_void_p(stream))
    N.check(rc)


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


@pytest.mark.parametrize("precision", [N.LFM_FP64, N.LFM_FP32_BULK], ids=["fp64", "fp32_bulk"])
@pytest.mark.parametrize("make", [
    lambda: cases.vortex_case(n=48, mu=1e-3),
    lambda: cases.cylinder_case(n_theta=64, n_r=32, r1=20, first=0.02, Ls=5, solver=2, minmod=True, noise=0.02),
    lambda: cases.cylinder_case(n_theta=24, n_r=12, r1=10, first=0.05, Ls=3, solver=1, n_span=6, noise=0.01),
])
def test_noalloc_residual_matches_regular_path_twice(make, precision):
    torch = pytest.importorskip("torch")
    case = make()
    case.residuals = True
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch, precision=precision)
    nq, nc = ch.desc.nq, ch.desc.n_cells
    stream = torch.cuda.current_stream().cuda_stream
    res_dev = torch.empty((nq, nc), dtype=torch.float64, device="cuda")
    q = ch.q0()
    for call in range(2):
        # regular path: the cell residual recorded at stage 0 of a step that
        # starts from q
        s.set_state(q)
        s.step(1, case.delta_t)
        s.sync()
        expected = s.cell_residual()
        # no-allocation path on the caller's buffers; the second call reads
        # its state from rows padded to nc + 17 values
        pad = 17 if call == 1 else 0
        host = np.zeros((nq, nc + pad))
        host[:, :nc] = q
        q_dev = torch.from_numpy(host).to("cuda")
        res_dev.fill_(float("nan"))
        _noalloc(s, q_dev, res_dev, stream)
        torch.cuda.synchronize()
        got = res_dev.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}"
        if precision == N.LFM_FP64:
            err = _rel(got, expected)
            assert np.all(err <= 1e-10), (call, err)
        else:
            scale = np.abs(expected).max(axis=1, keepdims=True)
            assert np.max(np.abs(got - expected) / scale) < 1e-4, call
        assert np.array_equal(q_dev.cpu().numpy(), host), "the state buffer must not be modified"
        q = s.get_state()   # the next call sees a different state


def test_noalloc_rejects_a_stride_below_the_cell_count():
    torch = pytest.importorskip("torch")
    case = cases.vortex_case(n=16)
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    q_dev = torch.from_numpy(ch.q0()).to("cuda")
    res_dev = torch.empty_like(q_dev)
    with pytest.raises(N.LfmError) as e:
        _noalloc(s, q_dev, res_dev, torch.cuda.current_stream().cuda_stream, stride=ch.desc.n_cells - 1)
    assert e.value.code == N.LFM_ERR_INVALID


def test_noalloc_rejects_a_partition_with_halos(tmp_path):
    torch = pytest.importorskip("torch")
    case = cases.vortex_case(n=24, solver=0)
    cases.decompose_case(case, str(tmp_path), 2)
    pc = N.PartitionedCase(str(tmp_path), 2)
    run = N.Partitioned(pc)
    h = C.c_void_p()
    N.check(N.load_library().lfm_partitioned_solver(run._h, 0, C.byref(h)))
    d = pc.descs[0]
    assert d.n_halos > 0
    q_dev = torch.from_numpy(pc.q0(0)).to("cuda")
    res_dev = torch.empty_like(q_dev)
    rc = N.load_library().lfm_solver_residual_noalloc(h, C.c_void_p(q_dev.data_ptr()), d.n_cells,
                                                      C.c_void_p(res_dev.data_ptr()),
                                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.LFM_ERR_UNSUPPORTED
    run.close()
    pc.close()


def test_noalloc_rejects_cases_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    case = cases.vortex_case(n=512)
    ch = N.CaseHandle.from_case(case)
    s = N.Solver(ch)
    q_dev = torch.from_numpy(ch.q0()).to("cuda")
    res_dev = torch.empty_like(q_dev)
    with pytest.raises(N.LfmError) as e:
        _noalloc(s, q_dev, res_dev, torch.cuda.current_stream().cuda_stream)
    assert e.value.code == -6 and "scratch" in str(e.value)
