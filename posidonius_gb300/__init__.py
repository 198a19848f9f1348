"""GB300-native WHFast + tidal-effects path of Posidonius (FP64, sm_103a).

Python mirror of the reference's integrator surface over the C ABI
(``include/posidonius_gb300.h``):

* :func:`restore_snapshot` -- ``output::restore_snapshot``
  (src/integrator/output.rs:178-203): open a WHFast JSON case, initialising
  the physical values of a new run;
* :class:`WHFast` -- one system, one kernel launch per step (the drop-in for
  ``WHFast`` + ``Integrator``, src/integrator/whfast.rs, src/integrator/mod.rs);
* :class:`Batch` -- many independent systems advanced by one persistent kernel
  replayed through a CUDA graph.

Nothing here computes physics on the CPU; every call goes to the CUDA library
and raises when it is missing.
"""
import ctypes

import numpy as np

from . import layout
from . import layout as L
from ._lib import PosiError, check, lib, ptr

__all__ = ["WHFast", "Batch", "ManyBody", "restore_snapshot", "read_case", "layout", "PosiError", "EXACT", "FAST"]

EXACT = L.MODE_EXACT
FAST = L.MODE_FAST

# output.rs:56-61 n_bytes_per_particle_in_historic_snapshot
HISTORY_BYTES_PER_PARTICLE = 8 + 8 + 4 + 8 * (20 - 3)


def read_case(path):
    """Parse a WHFast or IAS15 JSON case into the flat layout (C++ reader, no
    GPU); ``body_ias`` holds the IAS15 per-body state (zeros for WHFast)."""
    n = ctypes.c_int64()
    nt = ctypes.c_int64()
    check(lib().posi_read_case(str(path).encode(), ctypes.byref(n), ctypes.byref(nt), None, None, None, None, None,
                               None))
    n, nt = n.value, nt.value
    out = {
        "sys_i64": np.zeros(L.SI_COUNT, np.int64),
        "sys_f64": np.zeros(L.SF_COUNT, np.float64),
        "body_i64": np.zeros((n, L.BI_COUNT), np.int64),
        "body_f64": np.zeros((n, L.BF_COUNT), np.float64),
        "tables": np.zeros(max(nt, 1), np.float64),
        "roche": np.zeros((n, n), np.float64),
        "n": n,
    }
    check(lib().posi_read_case(str(path).encode(), None, None, ptr(out["sys_i64"], "i"), ptr(out["sys_f64"], "f"),
                               ptr(out["body_i64"], "i"), ptr(out["body_f64"], "f"), ptr(out["tables"], "f"),
                               ptr(out["roche"], "f")))
    if nt == 0:
        out["tables"] = np.zeros(1)
    out["body_ias"] = np.zeros((n, L.IAS_COUNT), np.float64)
    if out["sys_i64"][L.SI_INTEGRATOR] == L.INTEGRATOR_IAS15:
        check(lib().posi_read_case_ias15(str(path).encode(), ptr(out["body_ias"], "f")))
    return out


def _is_ias15(sys_i64):
    return int(np.asarray(sys_i64).reshape(-1, L.SI_COUNT)[0, L.SI_INTEGRATOR]) == L.INTEGRATOR_IAS15


class WHFast:
    """One system on the GPU (src/integrator/whfast.rs:99-1157; a case
    document of the IAS15 integrator, src/integrator/ias15.rs, steps by IAS15
    behind the same methods)."""

    def __init__(self, handle):
        if not handle:
            raise PosiError(L.ERR_ARG, "null handle")
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def from_json(cls, path, mode=EXACT):
        st = ctypes.c_int(0)
        h = lib().posi_universe_from_json(str(path).encode(), int(mode), ctypes.byref(st))
        if not h:
            check(st.value)
        return cls(h)

    @classmethod
    def from_arrays(cls, case, mode=EXACT):
        st = ctypes.c_int(0)
        arr = {k: np.ascontiguousarray(case[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64", "tables")}
        roche = case.get("roche")
        roche = None if roche is None else np.ascontiguousarray(roche, dtype=np.float64)
        h = lib().posi_universe_from_arrays(ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                            ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f"),
                                            ptr(arr["tables"], "f"), int(arr["tables"].size), ptr(roche, "f"),
                                            int(mode), ctypes.byref(st))
        if not h:
            check(st.value)
        w = cls(h)
        if _is_ias15(arr["sys_i64"]) and case.get("body_ias") is not None:
            ias = np.ascontiguousarray(case["body_ias"], dtype=np.float64)
            check(lib().posi_set_ias15(w._h, ptr(ias, "f")))
        return w

    def close(self):
        if self._h:
            lib().posi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # Integrator trait (src/integrator/mod.rs:16-27)
    def get_n_particles(self):
        n = ctypes.c_int64()
        check(lib().posi_get_n_particles(self._h, ctypes.byref(n)))
        return n.value

    def get_current_time(self):
        t = ctypes.c_double()
        check(lib().posi_get_current_time(self._h, ctypes.byref(t)))
        return t.value

    def get_n_historic_snapshots(self):
        n = ctypes.c_int64()
        check(lib().posi_get_n_historic_snapshots(self._h, ctypes.byref(n)))
        return n.value

    def set_time_limit(self, time_limit):
        check(lib().posi_set_time_limit(self._h, float(time_limit)))

    def set_snapshot_periods(self, historic_period, recovery_period):
        check(lib().posi_set_snapshot_periods(self._h, float(historic_period), float(recovery_period)))

    def initialize_physical_values(self):
        check(lib().posi_initialize_physical_values(self._h))

    def iterate(self, n_steps=1):
        """Advance up to n_steps steps.  Returns (status, steps_done, recovery_trigger);
        status is layout.OK or layout.COMPLETED ("Simulation completed")."""
        done = ctypes.c_int64()
        rec = ctypes.c_int()
        st = lib().posi_iterate(self._h, int(n_steps), ctypes.byref(done), ctypes.byref(rec))
        check(st, ok=(L.OK, L.COMPLETED))
        return st, done.value, bool(rec.value)

    def run(self, max_steps=None):
        """Iterate until the simulation completes or max_steps steps ran (the
        loop of src/main.rs:158-176 without snapshot writing).  Returns the
        number of steps performed."""
        total = 0
        while max_steps is None or total < max_steps:
            st, done, _ = self.iterate(10**9 if max_steps is None else max_steps - total)
            total += done
            if st == L.COMPLETED or done == 0:
                break
        return total

    # Snapshot output (src/integrator/output.rs)
    def open_history(self, path, expected_bytes=None):
        """get_universe_history_writer (output.rs:63-89): from now on every
        historic trigger appends its record to `path`.  expected_bytes
        defaults to n_historic_snapshots x 156 x n_particles."""
        if expected_bytes is None:
            expected_bytes = self.get_n_historic_snapshots() * HISTORY_BYTES_PER_PARTICLE * self.get_n_particles()
        check(lib().posi_open_history(self._h, str(path).encode(), int(expected_bytes)))

    def close_history(self):
        check(lib().posi_close_history(self._h))

    def write_recovery_snapshot(self, path):
        """WHFast::write_recovery_snapshot (whfast.rs:307-316): JSON snapshot
        of the current state; an existing file is kept as a dated backup."""
        check(lib().posi_write_recovery_snapshot(self._h, str(path).encode()))

    # Universe methods (src/particles/universe.rs)
    def gravity_calculate_acceleration(self, ignore_terms):
        check(lib().posi_gravity_calculate_acceleration(self._h, int(ignore_terms)))

    def calculate_additional_effects(self, current_time, evolution, dangular_momentum_dt, accelerations=True):
        check(lib().posi_calculate_additional_effects(self._h, float(current_time), int(bool(evolution)),
                                                      int(bool(dangular_momentum_dt)), int(bool(accelerations))))

    def get_state(self):
        n = self.get_n_particles()
        out = {
            "sys_i64": np.zeros(L.SI_COUNT, np.int64),
            "sys_f64": np.zeros(L.SF_COUNT, np.float64),
            "body_i64": np.zeros((n, L.BI_COUNT), np.int64),
            "body_f64": np.zeros((n, L.BF_COUNT), np.float64),
            "roche": np.zeros((n, n), np.float64),
            "n": n,
        }
        check(lib().posi_get_state(self._h, ptr(out["sys_i64"], "i"), ptr(out["sys_f64"], "f"),
                                   ptr(out["body_i64"], "i"), ptr(out["body_f64"], "f"), ptr(out["roche"], "f")))
        if _is_ias15(out["sys_i64"]):
            out["body_ias"] = np.zeros((n, L.IAS_COUNT), np.float64)
            check(lib().posi_get_ias15(self._h, ptr(out["body_ias"], "f")))
        return out

    def set_state(self, state):
        arr = {k: np.ascontiguousarray(state[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64")}
        check(lib().posi_set_state(self._h, ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                   ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f")))
        if _is_ias15(arr["sys_i64"]) and state.get("body_ias") is not None:
            ias = np.ascontiguousarray(state["body_ias"], dtype=np.float64)
            check(lib().posi_set_ias15(self._h, ptr(ias, "f")))


# a handle on an IAS15 case document
Ias15 = WHFast


def restore_snapshot(path, mode=EXACT):
    """src/integrator/output.rs:178-203: open a case; a new run (current_time 0)
    gets its physical values initialised."""
    w = WHFast.from_json(path, mode)
    if w.get_current_time() == 0.0:
        w.initialize_physical_values()
    return w


class Batch:
    """An ensemble of independent systems (flat layout, nmax bodies each)."""

    def __init__(self, ens, mode=FAST, mapping=L.MAP_AUTO):
        self.n_sys = int(ens["n_sys"])
        self.nmax = int(ens["nmax"])
        arr = {k: np.ascontiguousarray(ens[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64", "tables")}
        roche = ens.get("roche")
        roche = None if roche is None else np.ascontiguousarray(roche, dtype=np.float64)
        st = ctypes.c_int(0)
        h = lib().posi_batch_create(self.n_sys, self.nmax, ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                    ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f"), ptr(arr["tables"], "f"),
                                    int(arr["tables"].size), ptr(roche, "f"), int(mode), int(mapping),
                                    ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        self.ias15 = _is_ias15(arr["sys_i64"])
        if self.ias15 and ens.get("body_ias") is not None:
            ias = np.ascontiguousarray(ens["body_ias"], dtype=np.float64)
            check(lib().posi_batch_set_ias15(self._h, ptr(ias, "f")))

    def close(self):
        if self._h:
            lib().posi_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize_physical_values(self):
        check(lib().posi_batch_initialize_physical_values(self._h))

    def iterate(self, n_steps, steps_per_launch=0):
        check(lib().posi_batch_iterate(self._h, int(n_steps), int(steps_per_launch)))

    def set_balanced(self, on=True):
        """Balanced launch schedules on or off (posi_batch_set_balanced)."""
        check(lib().posi_batch_set_balanced(self._h, int(bool(on))))

    def last_timing(self):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        check(lib().posi_batch_last_timing(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def mapping_for(self, n):
        return lib().posi_batch_mapping_for(self._h, int(n))

    def autotune(self, probe_steps=20):
        """Pick the fastest lane mapping per body count (state unchanged).
        Returns {body count: lanes per system}."""
        out = (ctypes.c_int32 * (L.MAX_BODIES + 1))()
        check(lib().posi_batch_autotune(self._h, int(probe_steps), out))
        return {n: int(out[n]) for n in range(L.MAX_BODIES + 1) if out[n]}

    def autotune_report(self, n):
        """The last autotune's probe times (ms) for systems of n bodies, by
        lanes per system: {lanes: ms} for the mappings it tried."""
        ms = np.zeros(6, np.float64)
        check(lib().posi_batch_autotune_report(self._h, int(n), ptr(ms, "f")))
        return {1 << k: float(ms[k]) for k in range(6) if ms[k] >= 0}

    def empty_state(self):
        ns, nm = self.n_sys, self.nmax
        return {
            "sys_i64": np.zeros((ns, L.SI_COUNT), np.int64),
            "sys_f64": np.zeros((ns, L.SF_COUNT), np.float64),
            "body_i64": np.zeros((ns, nm, L.BI_COUNT), np.int64),
            "body_f64": np.zeros((ns, nm, L.BF_COUNT), np.float64),
            "roche": np.zeros((ns, nm, nm), np.float64),
            "n_sys": ns, "nmax": nm,
        }

    def get_state(self, out=None):
        out = out or self.empty_state()
        check(lib().posi_batch_get_state(self._h, ptr(out["sys_i64"], "i"), ptr(out["sys_f64"], "f"),
                                         ptr(out["body_i64"], "i"), ptr(out["body_f64"], "f"),
                                         ptr(out.get("roche"), "f")))
        if self.ias15:
            if out.get("body_ias") is None:
                out["body_ias"] = np.zeros((self.n_sys, self.nmax, L.IAS_COUNT), np.float64)
            check(lib().posi_batch_get_ias15(self._h, ptr(out["body_ias"], "f")))
        return out

    def set_state(self, state):
        arr = {k: np.ascontiguousarray(state[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64")}
        check(lib().posi_batch_set_state(self._h, ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                         ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f")))
        if self.ias15 and state.get("body_ias") is not None:
            ias = np.ascontiguousarray(state["body_ias"], dtype=np.float64)
            check(lib().posi_batch_set_ias15(self._h, ptr(ias, "f")))


class ManyBody:
    """One system of many bodies on the whole GPU (posi_large_*): WHFast in
    the case's coordinates (democratic heliocentric, Jacobi or WHDS), thread
    per body, the O(N^2) pair loop spread over every SM.  ``case`` is a
    single-system dict of the flat layout.  Tangents (``iterate_tangent``):
    democratic heliocentric only."""

    def __init__(self, case):
        st = ctypes.c_int(0)
        arr = {k: np.ascontiguousarray(case[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64")}
        self.n = int(arr["sys_i64"][L.SI_N])
        h = lib().posi_large_create(self.n, ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                    ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f"), ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)

    def close(self):
        if getattr(self, "_h", None):
            lib().posi_large_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize_physical_values(self):
        check(lib().posi_large_initialize_physical_values(self._h))

    def iterate(self, n_steps):
        """Returns layout.OK or layout.COMPLETED; raises on a physical event."""
        return check(lib().posi_large_iterate(self._h, int(n_steps)), ok=(L.OK, L.COMPLETED))

    def iterate_tangent(self, n_steps, seeds, tangents=None):
        """Forward-mode derivatives over n_steps (posi_large_iterate_tangent).

        ``seeds``: up to 4 directions, each ``(body, param)`` with param
        layout.SEED_SIGMA or layout.SEED_K2 (body -1: no parameter).
        ``tangents``: [len(seeds), n, 12] initial state tangents (r, v, L, S
        per body), zeros when None.  Returns (status, tangents after the
        steps): d state / d parameter for a pure parameter seed."""
        nd = len(seeds)
        body = np.ascontiguousarray([int(b) for b, _ in seeds], dtype=np.int32)
        param = np.ascontiguousarray([int(p) for _, p in seeds], dtype=np.int32)
        tan = np.zeros((nd, self.n, 12), np.float64) if tangents is None else \
            np.array(tangents, dtype=np.float64, order="C").reshape(nd, self.n, 12)
        rc = check(lib().posi_large_iterate_tangent(self._h, int(n_steps), nd, ptr(body, "i32"), ptr(param, "i32"),
                                                    ptr(tan, "f")), ok=(L.OK, L.COMPLETED))
        return rc, tan

    def last_timing(self):
        ms = ctypes.c_double()
        check(lib().posi_large_last_timing(self._h, ctypes.byref(ms)))
        return ms.value

    def get_state(self):
        n = self.n
        out = {"sys_i64": np.zeros(L.SI_COUNT, np.int64), "sys_f64": np.zeros(L.SF_COUNT, np.float64),
               "body_i64": np.zeros((n, L.BI_COUNT), np.int64), "body_f64": np.zeros((n, L.BF_COUNT), np.float64),
               "n": n}
        check(lib().posi_large_get_state(self._h, ptr(out["sys_i64"], "i"), ptr(out["sys_f64"], "f"),
                                         ptr(out["body_i64"], "i"), ptr(out["body_f64"], "f")))
        return out

    def set_state(self, state):
        arr = {k: np.ascontiguousarray(state[k], dtype=np.int64 if k.endswith("i64") else np.float64)
               for k in ("sys_i64", "sys_f64", "body_i64", "body_f64")}
        check(lib().posi_large_set_state(self._h, ptr(arr["sys_i64"], "i"), ptr(arr["sys_f64"], "f"),
                                         ptr(arr["body_i64"], "i"), ptr(arr["body_f64"], "f")))


# the pure-Python parts: seeded systems and ensembles, case documents
from . import case_writer, ensemble  # noqa: E402,F401
