"""GPU: the allocation-free adjoint entry point (posi_adjoint_vjp_static).

Called through the C ABI with device arrays the test owns (torch CUDA
tensors in the library's field-major layout), it must give the same adjoints
and parameter gradients as the allocating entry point
(posi_adjoint_create / _forward / _backward, one chunk) on the same state --
on two calls in a row with different adjoint seeds, so that the shared
static scratch carries nothing from one call to the next.
"""
import ctypes

import numpy as np
import pytest

import posidonius_gb300 as pg
from posidonius_gb300 import adjoint as A, layout as L
from posidonius_gb300._lib import lib

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative; the two paths run the same kernels on the same inputs


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _field_major(torch, a, dtype):
    """[rows, fields] (host layout) -> contiguous [fields, rows] on the GPU."""
    a = np.ascontiguousarray(np.asarray(a).reshape(-1, a.shape[-1]).T)
    return torch.tensor(a, dtype=dtype, device="cuda").contiguous()


def test_static_adjoint_matches_allocating_adjoint_twice():
    torch = pytest.importorskip("torch")
    n_steps = 30
    ens, el, ms, moi, ss = A.gradient_workload(12, seed=5)
    # an EXACT batch: its backward pass re-integrates with the adjoint's own
    # forward, as the allocation-free entry point does
    batch = pg.Batch(ens, mode=pg.EXACT)
    batch.initialize_physical_values()
    state = batch.get_state()
    ns, nm = batch.n_sys, batch.nmax
    adj = A.Adjoint(batch, n_steps, n_steps)
    adj.forward()
    si = _field_major(torch, state["sys_i64"], torch.int64)
    sf = _field_major(torch, state["sys_f64"], torch.float64)
    bi = _field_major(torch, state["body_i64"], torch.int64)
    bf = _field_major(torch, state["body_f64"], torch.float64)
    rng = np.random.default_rng(0)
    for call in range(2):
        lam = rng.normal(size=(ns, nm, 12))
        ref_lam, ref_grad = adj.backward(lam.copy())
        assert not adj.flags.any()
        d_lam = _field_major(torch, lam, torch.float64)
        d_grad = torch.zeros((2, ns * nm), dtype=torch.float64, device="cuda")
        d_flags = torch.full((ns,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib().posi_adjoint_vjp_static(ns, nm, si.data_ptr(), sf.data_ptr(), bi.data_ptr(), bf.data_ptr(),
                                           n_steps, d_lam.data_ptr(), d_grad.data_ptr(), d_flags.data_ptr(), None)
        assert rc == L.OK, lib().posi_last_error()
        torch.cuda.synchronize()
        assert (d_flags.cpu().numpy() == 0).all()
        got_lam = d_lam.cpu().numpy().T.reshape(ns, nm, 12)
        got_grad = d_grad.cpu().numpy().T.reshape(ns, nm, 2)
        for got, ref in ((got_lam, ref_lam), (got_grad, ref_grad)):
            scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
            assert (np.abs(got - ref) <= TOL * scale).all(), (call, np.abs(got - ref).max())


def test_static_adjoint_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    ens, el, ms, moi, ss = A.gradient_workload(4, seed=5)
    batch = pg.Batch(ens, mode=pg.FAST)
    batch.initialize_physical_values()
    state = batch.get_state()
    ns, nm = batch.n_sys, batch.nmax
    si = _field_major(torch, state["sys_i64"], torch.int64)
    sf = _field_major(torch, state["sys_f64"], torch.float64)
    bi = _field_major(torch, state["body_i64"], torch.int64)
    bf = _field_major(torch, state["body_f64"], torch.float64)
    d_lam = torch.zeros((12, ns * nm), dtype=torch.float64, device="cuda")
    d_grad = torch.zeros((2, ns * nm), dtype=torch.float64, device="cuda")
    d_flags = torch.zeros((ns,), dtype=torch.int32, device="cuda")
    rc = lib().posi_adjoint_vjp_static(ns, nm, si.data_ptr(), sf.data_ptr(), bi.data_ptr(), bf.data_ptr(), 10 ** 6,
                                       d_lam.data_ptr(), d_grad.data_ptr(), d_flags.data_ptr(), None)
    assert rc == L.ERR_ARG
    assert b"static scratch" in lib().posi_last_error()
