"""The allocation-free direct sum, gb_direct_accel_noalloc.

Some callers cannot allocate GPU memory: hosts that own every device
allocation through their own pool, runtimes that forbid cudaMalloc once they
run, plugins that may only use the buffers they are given. This test acts as
such a caller: its device buffers come from its own allocator (torch), and the
library call allocates nothing. The result must equal that of the
context-based entry point gb_direct_accel on the same input within the
relative tolerance the direct-sum tests use (1e-13), on two calls in a row
(the second call reuses the scratch array the first one left behind), and the
second call must not change the device's free memory.

The file name makes pytest collect it last, so a failure here cannot keep a
`-x` run from running every other test first.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13


def rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def test_noalloc_direct_sum_matches_context_entry_point():
    import torch

    import vipp_gb300

    lib = vipp_gb300.load()
    n, eps, G = 6000, 0.01, 1.0
    m = 1.0 / n
    x, _ = O.plummer_reference(n, eps, 11)
    rng = np.random.default_rng(4)
    target_sets = [np.sort(rng.choice(n, 1500, replace=False)), np.sort(rng.choice(n, 777, replace=False))]

    with vipp_gb300.Solver(p=4, s=8, eps=eps, G=G, m=m) as ctx:
        ctx.preprocess(x, np.zeros_like(x))
        expected = [ctx.direct_accel(t) for t in target_sets]

    dev = torch.device("cuda", 0)
    x_dev = torch.from_numpy(x).to(dev)
    stream = torch.cuda.current_stream(dev)
    free_after = []
    for t, want in zip(target_sets, expected):
        t_dev = torch.from_numpy(t.astype(np.int64)).to(dev)
        a_dev = torch.full((len(t), 3), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        rc = lib.gb_direct_accel_noalloc(x_dev.data_ptr(), n, t_dev.data_ptr(), len(t), G, m, eps, a_dev.data_ptr(),
                                         stream.cuda_stream)
        assert rc == vipp_gb300.GB_OK
        torch.cuda.synchronize(dev)
        free_after.append(torch.cuda.mem_get_info(dev)[0])
        got = a_dev.cpu().numpy()
        assert np.max(rel(got, want)) <= TOL
        assert np.max(rel(got, O.direct_accel(x, G, m, eps, t))) <= TOL
    assert free_after[1] == free_after[0]  # the second call allocated nothing


def test_noalloc_all_particles_and_out_of_range_targets():
    """targets_dev = NULL computes every particle (against the oracle's sum
    over all particles); indices outside [0, n) give NaN rows, the valid ones
    their sums; a target list with n == 0 is rejected."""
    import torch

    import vipp_gb300

    lib = vipp_gb300.load()
    n, eps, G = 3000, 0.01, 1.0
    m = 1.0 / n
    x, _ = O.plummer_reference(n, eps, 12)
    dev = torch.device("cuda", 0)
    x_dev = torch.from_numpy(x).to(dev)
    a_dev = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    assert lib.gb_direct_accel_noalloc(x_dev.data_ptr(), n, None, 0, G, m, eps, a_dev.data_ptr(), None) == 0
    torch.cuda.synchronize(dev)
    assert np.max(rel(a_dev.cpu().numpy(), O.direct_accel(x, G, m, eps))) <= TOL
    t = np.array([-1, n, 5], dtype=np.int64)
    t_dev = torch.from_numpy(t).to(dev)
    b_dev = torch.zeros((3, 3), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    assert lib.gb_direct_accel_noalloc(x_dev.data_ptr(), n, t_dev.data_ptr(), 3, G, m, eps, b_dev.data_ptr(), None) == 0
    torch.cuda.synchronize(dev)
    b = b_dev.cpu().numpy()
    assert np.all(np.isnan(b[0])) and np.all(np.isnan(b[1]))
    assert np.max(rel(b[2:], O.direct_accel(x, G, m, eps, np.array([5])))) <= TOL
    rc = lib.gb_direct_accel_noalloc(x_dev.data_ptr(), 0, t_dev.data_ptr(), 3, G, m, eps, b_dev.data_ptr(), None)
    assert rc == vipp_gb300.GB_ERR_INVALID


def test_noalloc_rejects_more_targets_than_its_scratch_holds():
    import torch

    import vipp_gb300

    lib = vipp_gb300.load()
    dev = torch.device("cuda", 0)
    x_dev = torch.zeros((10, 3), dtype=torch.float64, device=dev)
    t_dev = torch.zeros(1, dtype=torch.int64, device=dev)
    a_dev = torch.zeros((1, 3), dtype=torch.float64, device=dev)
    rc = lib.gb_direct_accel_noalloc(x_dev.data_ptr(), 10, t_dev.data_ptr(), 699051, 1.0, 1.0, 0.01, a_dev.data_ptr(),
                                     None)
    assert rc == vipp_gb300.GB_ERR_CAPACITY
