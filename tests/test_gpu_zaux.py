"""Auxiliary entry points on the GPU: the JSON solve log (one record per
solve, the numbers of the reference's solver report line) and the
multi-field download used before a restart dump."""
import json

import numpy as np
import pytest

from cd_cases import cd_batch_system
from conftest import load_fcgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def actx():
    fc = load_fcgpu()
    c = fc.Context(0)
    yield fc, c
    c.close()


def test_solve_log_records_each_solve(actx, tmp_path):
    fc, c = actx
    probs = [cd_batch_system(fc, c, n, 1.0, seed=200 + n) for n in (8, 10)]
    log = tmp_path / "solves.jsonl"
    c.set_solve_log(str(log))
    try:
        ia, ja, dg, a, b, _ = probs[0]
        x, _, info, st = c.csrsolve("bicgstab", ia, ja, a, dg, np.zeros(len(dg)), b, 500, 0.0, 1e-8, chvar="T")
        B = fc.Batch(c)
        for ia_, ja_, dg_, _, _, xyz in probs:
            B.add(ia_, ja_, dg_, xyz)
        B.plan()
        _, binfos, _ = B.solve([p[3] for p in probs], [np.zeros(len(p[2])) for p in probs], [p[4] for p in probs],
                               500, 0.0, 1e-8)
        B.close()
    finally:
        c.set_solve_log(None)
    rec = [json.loads(line) for line in open(log)]
    assert len(rec) == 3
    assert rec[0]["api"] == "fc_csrsolve" and rec[0]["solver"] == "bicgstab" and rec[0]["var"] == "T"
    assert rec[0]["n"] == len(probs[0][2]) and rec[0]["status"] == st
    assert rec[0]["iterations"] == info.itr_used
    assert rec[0]["resl"] == info.resl and rec[0]["res0_l1"] == info.res0_l1 and rec[0]["resor"] == info.resor
    for k in (0, 1):
        r = rec[1 + k]
        assert r["api"] == "fc_batch_solve" and r["var"] == f"problem {k}"
        assert r["iterations"] == binfos[k].itr_used and r["resl"] == binfos[k].resl


def test_download_fields_matches_field_get(actx):
    fc, c = actx
    cd_batch_system(fc, c, 9, 2.0, seed=7)
    c.field_set("dPdxi", np.arange(c.field_len("dPdxi"), dtype=np.float64))
    names = ["su", "flmass", "dPdxi", "a"]
    got = c.download_fields(names)
    for nm in names:
        assert np.array_equal(got[nm], c.field_get(nm)), nm
