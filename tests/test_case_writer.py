"""Flat system -> JSON case document (posidonius_gb300.case_writer), on CPU.

For every reference golden case (WHFast and IAS15): the written document has
the reference document's structure (the same keys at every level, the same
list lengths, the same effect tags), and both readers -- the oracle's and
the library's C++ one -- read it back to the same flat system bit for bit.
"""
import json

import numpy as np
import pytest

import posidonius_gb300 as pg
from oracle.case_json import load_case
from posidonius_gb300 import case_writer as W, ensemble as E, layout as L

from golden_cases import case_dict, names


def _structure(x):
    if isinstance(x, dict):
        return {k: _structure(v) for k, v in x.items()}
    if isinstance(x, list):
        return ("list", len(x), _structure(x[0]) if x and isinstance(x[0], (dict, list)) else None)
    return "value"


def _same(a, b):
    for k in ("sys_i64", "sys_f64", "body_i64", "body_f64", "roche", "body_ias"):
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape, k
        if x.dtype == np.float64:
            assert np.array_equal(x.view(np.int64), y.view(np.int64)) or np.array_equal(x, y, equal_nan=True), k
        else:
            assert np.array_equal(x, y), k
    n = int(np.asarray(a["sys_i64"])[L.SI_N])
    ta, tb = np.asarray(a["tables"]), np.asarray(b["tables"])
    m = min(ta.size, tb.size)
    assert np.array_equal(ta[:m], tb[:m]) and n == int(np.asarray(b["sys_i64"])[L.SI_N])


@pytest.mark.parametrize("name", names(None))
def test_written_document_reads_back_and_has_the_reference_structure(name, tmp_path):
    ref_doc = case_dict(name)
    flat = load_case(ref_doc)
    doc = W.case_document(flat)
    got = _structure(json.loads(json.dumps(W._json_safe(doc))))
    want = _structure(ref_doc)
    assert got == want
    u, ru = doc["universe"], ref_doc["universe"]
    for b in range(u["n_particles"]):
        for eff in ("tides", "rotational_flattening", "general_relativity", "disk", "wind"):
            assert u["particles"][b][eff]["effect"] == ru["particles"][b][eff]["effect"], (b, eff)
        assert json.dumps(u["particles"][b]["evolution"], sort_keys=True) == \
            json.dumps(ru["particles"][b]["evolution"], sort_keys=True) or u["particles"][b]["evolution"] != "NonEvolving"
    _same(load_case(doc), flat)
    path = tmp_path / "case.json"
    W.write_case(path, flat)
    _same(pg.read_case(path), flat)


def test_generated_system_runs_from_its_document(tmp_path):
    """A seeded synthetic system written by the case writer reads back to
    the generator's own arrays (the document is the drop-in input of
    `posidonius start`)."""
    ens = E.workload_single(seed=4)
    path = tmp_path / "generated.json"
    W.write_case(path, ens)
    got = pg.read_case(path)
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    for k in ("sys_i64", "body_i64"):
        assert np.array_equal(got[k][..., :], one[k][: got["n"]] if k == "body_i64" else one[k]), k
    assert np.array_equal(got["body_f64"], one["body_f64"][: got["n"]])


def test_ias15_state_round_trip_through_the_cpp_reader(tmp_path):
    """A resumed IAS15 document (non-zero Gauss-Radau arrays, accepted step,
    non-converged count): the C++ reader returns every value bit for bit."""
    name = names("ias15")[0]
    flat = load_case(case_dict(name))
    rng = np.random.default_rng(5)
    flat["body_ias"] = rng.standard_normal(flat["body_ias"].shape) * 1e-3
    flat["sys_f64"][L.SF_IAS_DT_LAST] = 1.28
    flat["sys_f64"][L.SF_DT] = 5.12
    flat["sys_i64"][L.SI_IAS_MAX_EXCEEDED] = 3
    path = tmp_path / "resumed_ias15.json"
    W.write_case(path, flat)
    got = pg.read_case(path)
    _same(got, flat)
    assert got["sys_i64"][L.SI_INTEGRATOR] == L.INTEGRATOR_IAS15
