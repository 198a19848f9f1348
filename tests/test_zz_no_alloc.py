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
from posidonius_gb300 import adjoint as A, ensemble as E, layout as L
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
    for n_steps in (10 ** 6, 2 ** 62, 2 ** 63 - 1):
        # 2**62 steps would wrap a size computed by multiplication first
        rc = lib().posi_adjoint_vjp_static(ns, nm, si.data_ptr(), sf.data_ptr(), bi.data_ptr(), bf.data_ptr(),
                                           n_steps, d_lam.data_ptr(), d_grad.data_ptr(), d_flags.data_ptr(), None)
        assert rc == L.ERR_ARG, n_steps
        assert b"static scratch" in lib().posi_last_error()


def _static_call(torch, si, sf, bi, bf, ns, nm, n_steps, lam, grad):
    d_lam = lam.clone()
    d_grad = grad.clone()
    d_flags = torch.full((ns,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib().posi_adjoint_vjp_static(ns, nm, si.data_ptr(), sf.data_ptr(), bi.data_ptr(), bf.data_ptr(), n_steps,
                                       d_lam.data_ptr(), d_grad.data_ptr(), d_flags.data_ptr(), None)
    assert rc == L.OK, lib().posi_last_error()
    torch.cuda.synchronize()
    return d_lam.cpu().numpy(), d_grad.cpu().numpy(), d_flags.cpu().numpy()


def test_static_adjoint_leaves_unsupported_systems_out():
    """Systems the adjoint does not support get POSI_ADJ_UNSUPPORTED and are
    left out of the run: their adjoints and gradients stay as they were, and
    their neighbours' results are those of a run without them.  With three
    bodies per system the kernels use groups of four lanes, so a system that
    claims four bodies would reach into the next system's (or, for the last
    one, past the arrays') bodies if it were run."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    ens = E.stack_systems([E.system_single(rng, n_planets=2) for _ in range(6)])
    batch = pg.Batch(ens, mode=pg.EXACT)
    batch.initialize_physical_values()
    state = batch.get_state()
    ns, nm = batch.n_sys, batch.nmax
    assert nm == 3
    si_host = np.array(state["sys_i64"])
    sf = _field_major(torch, state["sys_f64"], torch.float64)
    bi = _field_major(torch, state["body_i64"], torch.int64)
    bf = _field_major(torch, state["body_f64"], torch.float64)
    lam = _field_major(torch, rng.normal(size=(ns, nm, 12)), torch.float64)
    grad = _field_major(torch, rng.normal(size=(ns, nm, 2)), torch.float64)
    n_steps = 12
    ref_lam, ref_grad, ref_flags = _static_call(torch, _field_major(torch, si_host, torch.int64), sf, bi, bf, ns, nm,
                                                n_steps, lam, grad)
    assert (ref_flags == 0).all()
    bad = si_host.copy()
    bad[1, L.SI_COORDS] = L.DEMOCRATIC_HELIOCENTRIC
    bad[3, L.SI_N] = 4
    bad[5, L.SI_N] = 4
    got_lam, got_grad, flags = _static_call(torch, _field_major(torch, bad, torch.int64), sf, bi, bf, ns, nm, n_steps,
                                            lam, grad)
    left_out, kept = [1, 3, 5], [0, 2, 4]
    assert (flags[left_out] == L.ADJ_UNSUPPORTED).all() and (flags[kept] == 0).all()
    lam0, grad0 = lam.cpu().numpy(), grad.cpu().numpy()
    for s in range(ns):
        cols = slice(s * nm, (s + 1) * nm)
        want_lam, want_grad = (lam0, grad0) if s in left_out else (ref_lam, ref_grad)
        assert np.array_equal(got_lam[:, cols], want_lam[:, cols]), s
        assert np.array_equal(got_grad[:, cols], want_grad[:, cols]), s
