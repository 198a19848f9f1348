"""Comparison helpers shared by the parity tests."""
import numpy as np

from posidonius_gb300 import layout as L

# every body field is state the kernels maintain (the tidal dE/dt is refreshed
# at historic-snapshot steps and is NaN after the first one, 0/0)
STATE_FIELDS = list(range(L.BF_COUNT))
SYS_I64_FIELDS = [L.SI_ITERATION, L.SI_N_HIST, L.SI_TIMESTEP_WARNING, L.SI_STATUS, L.SI_FAIL_STEP, L.SI_FAIL_PAIR,
                  L.SI_LAST_MIDPOINT_ITERS, L.SI_IAS_MAX_EXCEEDED]
# the IAS15 step size adapts (constant for WHFast)
SYS_F64_FIELDS = [L.SF_TIME, L.SF_LAST_HIST, L.SF_LAST_REC, L.SF_DT, L.SF_IAS_DT_LAST]


def nbodies(ens, s):
    return int(ens["sys_i64"][s, L.SI_N]) if ens["sys_i64"].ndim == 2 else int(ens["sys_i64"][L.SI_N])


def as_batch_view(state):
    """Promote a single-system state (2-D body arrays) to ensemble shape."""
    if state["body_f64"].ndim == 2:
        return {k: (v[None] if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    return state


def same_bits(fa, fb):
    """Element-wise: identical bits, or both NaN (the NaN payload of 0/0
    differs between host architectures and the GPU)."""
    fa, fb = np.asarray(fa, dtype=np.float64), np.asarray(fb, dtype=np.float64)
    return (fa.view(np.int64) == fb.view(np.int64)) | (np.isnan(fa) & np.isnan(fb))


def bitwise_diffs(a, b):
    """Fields whose values differ in any bit (NaN matching NaN); [] when identical."""
    a, b = as_batch_view(a), as_batch_view(b)
    out = []
    ns = a["sys_i64"].shape[0]
    for s in range(ns):
        n = nbodies(a, s)
        fa, fb = a["body_f64"][s, :n][:, STATE_FIELDS], b["body_f64"][s, :n][:, STATE_FIELDS]
        same = same_bits(fa, fb)
        if not same.all():
            bad = np.nonzero((~same).any(axis=0))[0]
            out.append((s, "body_f64", [STATE_FIELDS[i] for i in bad]))
        if not np.array_equal(a["body_i64"][s, :n, L.BI_EVO_LEFT], b["body_i64"][s, :n, L.BI_EVO_LEFT]):
            out.append((s, "evo_left", None))
        for f in SYS_I64_FIELDS:
            if a["sys_i64"][s, f] != b["sys_i64"][s, f]:
                out.append((s, "sys_i64", f))
        for f in SYS_F64_FIELDS:
            if not same_bits(a["sys_f64"][s, f], b["sys_f64"][s, f]):
                out.append((s, "sys_f64", f))
        if a.get("body_ias") is not None and b.get("body_ias") is not None:
            same = same_bits(a["body_ias"][s, :n], b["body_ias"][s, :n])
            if not same.all():
                out.append((s, "body_ias", list(np.nonzero((~same).any(axis=0))[0])))
    return out


def max_rel_error(a, b, fields=(L.POS, L.VEL, L.ANG)):
    """Largest |a-b| / max|b| per vector quantity over all systems and bodies."""
    a, b = as_batch_view(a), as_batch_view(b)
    worst = 0.0
    for s in range(a["sys_i64"].shape[0]):
        n = nbodies(a, s)
        for sl in fields:
            va, vb = a["body_f64"][s, :n, sl], b["body_f64"][s, :n, sl]
            scale = np.abs(vb).max()
            if scale > 0:
                worst = max(worst, float(np.abs(va - vb).max() / scale))
    return worst
