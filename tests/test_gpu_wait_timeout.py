"""A bounded device wait that runs out is reported, never passed over as a
success: the kernel records it (a device counter and a host-mapped word),
and the next call that launches FFT work on the device returns
MDFT_ERR_TIMEOUT with a message (the reference reports every failure by
Throw_If, common/MDFT_Asserts.hpp:15-28).  The timeout is made on purpose by
a one-CTA kernel waiting on a barrier that nothing completes, with a short
poll limit -- no fault and no hang."""
import pytest

from mini_mdft_gb300 import inputs as I

pytestmark = pytest.mark.gpu


def test_timed_out_wait_fails_the_next_call_once(gpu_lib):
    import torch
    M = gpu_lib
    n, box, mmax, mrso, dq = (32, 32, 32), (20., 20., 20.), 3, 2, 0.01
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, dq), dq)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    conv = M.Convolution.from_table(idx, tab, dq, sg, ag, precision="f64df")
    g = torch.Generator(device="cuda").manual_seed(5)
    p = torch.randn((ag.m_np,) + n, generator=g, device="cuda", dtype=torch.complex128)
    ref = p.clone()
    conv.execute(ref)
    torch.cuda.synchronize()
    before = M.wait_timeouts()

    M.wait_selftest(256)
    torch.cuda.synchronize()
    assert M.wait_timeouts() == before + 1
    q = p.clone()
    with pytest.raises(M.MdftError) as e:
        conv.execute(q)
    assert e.value.code == 6
    assert "wait ran out" in str(e.value)
    # reported once: the call after it runs, and gives the usual result
    conv.execute(q)
    torch.cuda.synchronize()
    assert torch.equal(q, ref)


def test_persistent_kernel_barrier_timeout_is_reported(gpu_lib):
    """The grid barrier of the persistent L-BFGS kernel: with every block
    present it passes; with one arrival missing every block gives up (bounded
    poll), the timeout is counted, and the next convolution call returns
    MDFT_ERR_TIMEOUT once."""
    import torch
    M = gpu_lib
    n, box, mmax, mrso, dq = (16, 16, 16), (10., 10., 10.), 2, 2, 0.01
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, dq), dq)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    conv = M.Convolution.from_table(idx, tab, dq, sg, ag, precision="f64")
    p = torch.zeros((ag.m_np,) + n, device="cuda", dtype=torch.complex128)
    before = M.wait_timeouts()
    M.grid_barrier_selftest(0)
    torch.cuda.synchronize()
    assert M.wait_timeouts() == before
    conv.execute(p)
    M.grid_barrier_selftest(1)
    torch.cuda.synchronize()
    assert M.wait_timeouts() == before + 1
    with pytest.raises(M.MdftError) as e:
        conv.execute(p)
    assert e.value.code == 6
    conv.execute(p)
    torch.cuda.synchronize()
