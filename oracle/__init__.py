"""CPU oracle for the WHFast + tidal-effects path (test infrastructure only).

``whfast_oracle.cpp`` restates the reference's Rust FP64 functions in C++ in
the same operation order; ``case_json.py`` reads the reference's JSON cases.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
load this package -- as the checker and the CPU baseline, never as the
measured product path.
"""
import ctypes
import os
import subprocess

import numpy as np

from posidonius_gb300 import layout as L

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_FLOPS = os.path.join(BUILD, "liboracle_flops.so")
LIB_DUAL = os.path.join(BUILD, "liboracle_dual.so")

ITERATE, GRAVITY, ADDITIONAL_EFFECTS, INITIALIZE = 0, 1, 2, 3


def build(force=False):
    """Compile the oracle with make (g++, -ffp-contract=off)."""
    if force or not (os.path.exists(LIB) and os.path.exists(LIB_FLOPS)):
        subprocess.check_call(["make", "-s", "-C", HERE, "-j2"])
    else:
        subprocess.check_call(["make", "-s", "-C", HERE, "-j2"])


_libs = {}


def _lib(flops=False, dual=False):
    path = LIB_FLOPS if flops else LIB_DUAL if dual else LIB
    if path not in _libs:
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        i64p = ctypes.POINTER(ctypes.c_int64)
        f64p = ctypes.POINTER(ctypes.c_double)
        lib.oracle_run.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, i64p, f64p, i64p, f64p, f64p,
                                   f64p, f64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_int, i64p, i64p]
        lib.oracle_run.restype = ctypes.c_int
        lib.oracle_history.argtypes = [f64p, ctypes.c_int64, i64p]
        lib.oracle_history.restype = None
        lib.oracle_constant.argtypes = [ctypes.c_int]
        lib.oracle_constant.restype = ctypes.c_double
        if flops:
            lib.oracle_flops.argtypes = [i64p, ctypes.c_int]
        if dual:
            lib.oracle_dual_io.argtypes = [f64p, f64p]
            lib.oracle_dual_io.restype = ctypes.c_int
        _libs[path] = lib
    return _libs[path]


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def as_ensemble(case):
    """Accept a single-system dict (case_json.load_case) or a stacked ensemble."""
    if "n_sys" in case:
        return case
    from .case_json import stack
    return stack([case])


def run_with_history(case, max_steps, init_physical=False, max_records=100000):
    """ITERATE one system single-threaded, collecting its historic records.

    Returns (ensemble, steps_done, result, records) with records an array of
    shape (n_triggers, n_bodies, 20) in the kernel's record layout.
    """
    lib = _lib()
    ens = as_ensemble(case)
    if ens["n_sys"] != 1:
        raise ValueError("run_with_history takes one system")
    n = int(ens["sys_i64"][0, L.SI_N])
    buf = np.zeros((max_records, 20), dtype=np.float64)
    length = np.zeros(1, dtype=np.int64)
    lib.oracle_history(_p(buf, ctypes.c_double), max_records, None)
    try:
        out = run(ens, max_steps=max_steps, init_physical=init_physical, nthreads=1)
        lib.oracle_history(_p(buf, ctypes.c_double), max_records, _p(length, ctypes.c_int64))
    finally:
        lib.oracle_history(None, 0, None)
    k = int(length[0])
    return out + (buf[:k].reshape(k // n, n, 20),)


def run(ens, op=ITERATE, max_steps=0, init_physical=False, arg=0, t_arg=0.0, nthreads=1, flops=False,
        _dual_lib=None):
    """Run `op` in place on a copy of the ensemble; returns (ensemble, steps_done, result[, flops])."""
    ens = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in as_ensemble(ens).items()}
    lib = _dual_lib or _lib(flops)
    ns, nmax = ens["n_sys"], ens["nmax"]
    if "body_ias" not in ens:
        ens["body_ias"] = np.zeros((ns, nmax, L.IAS_COUNT))
    for k, dt in (("sys_i64", np.int64), ("sys_f64", np.float64), ("body_i64", np.int64),
                  ("body_f64", np.float64), ("tables", np.float64), ("roche", np.float64),
                  ("body_ias", np.float64)):
        ens[k] = np.ascontiguousarray(ens[k], dtype=dt)
    steps = np.zeros(ns, dtype=np.int64)
    result = np.zeros(ns, dtype=np.int64)
    if flops:
        cnt = np.zeros(3, dtype=np.int64)
        lib.oracle_flops(_p(cnt, ctypes.c_int64), 1)
    lib.oracle_run(op, ns, nmax, _p(ens["sys_i64"], ctypes.c_int64), _p(ens["sys_f64"], ctypes.c_double),
                   _p(ens["body_i64"], ctypes.c_int64), _p(ens["body_f64"], ctypes.c_double),
                   _p(ens["tables"], ctypes.c_double), _p(ens["roche"], ctypes.c_double),
                   _p(ens["body_ias"], ctypes.c_double), int(max_steps),
                   int(init_physical), int(arg), float(t_arg), 1 if flops else int(nthreads),
                   _p(steps, ctypes.c_int64), _p(result, ctypes.c_int64))
    if flops:
        lib.oracle_flops(_p(cnt, ctypes.c_int64), 1)
        return ens, steps, result, cnt
    return ens, steps, result


def constant(which):
    return _lib().oracle_constant(which)


def dual_directions():
    """Directional derivatives every value of the dual build carries."""
    return _lib(dual=True).oracle_dual_io(None, None)


def run_dual(ens, seed, max_steps, init_physical=False, nthreads=1):
    """ITERATE with forward-mode dual numbers: the exact derivatives of the
    oracle's computed map (its operation order, its branches) along the
    seeded directions.  seed [n_sys, nmax, BF_COUNT, ND]: derivatives of the
    inputs (position, velocity, spin angular momentum, spin, dissipation
    factor, Love number of each body) along each direction.  Returns
    (ensemble, steps_done, result, tangents [n_sys, nmax, BF_COUNT, ND]) --
    tangents of the final position, velocity, spin angular momentum and
    spin (other fields zero)."""
    lib = _lib(dual=True)
    ens = as_ensemble(ens)
    nd = lib.oracle_dual_io(None, None)
    shape = (int(ens["n_sys"]), int(ens["nmax"]), L.BF_COUNT, nd)
    seed = np.ascontiguousarray(np.broadcast_to(seed, shape), dtype=np.float64)
    out = np.zeros(shape, dtype=np.float64)
    lib.oracle_dual_io(_p(seed, ctypes.c_double), _p(out, ctypes.c_double))
    try:
        res = run(ens, max_steps=max_steps, init_physical=init_physical, nthreads=nthreads, _dual_lib=lib)
    finally:
        lib.oracle_dual_io(None, None)
    return res + (out,)
