"""The oracle against the reference's own operator unit tests, driven by the
fixture tests/golden/known_answers.json (extracted from the reference's test
sources by tests/golden/make_known_answers.py): each test's input tables,
built as the reference test builds them, give the count it asserts."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import bool_to_words

FIXTURE = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())
VAR_IDS = {}


def var_id(name):
    return VAR_IDS.setdefault(name, len(VAR_IDS) + 1)


def table(dep):
    names = [c for c, _ in dep["schema"]]
    var = [var_id(n) for n in names]
    vec = dep["vectors"]
    if dep["kind"] == "Flat":
        cols = []
        for (col, typ), vname in zip(dep["schema"], list(vec)[:2]):
            cols.append(np.asarray(vec[vname], np.int64 if typ == "Int64" else np.uint32))
        return O.Table(O.FLAT, var, cols=cols)
    rows, ncols = dep["shape"]
    rv, kv = vec[dep["set"]["row"]], vec[dep["set"]["col_key"]]
    k_map = {}
    for x in kv:  # columns in order of first appearance, as the reference test builds them
        k_map.setdefault(x, len(k_map))
    m = np.zeros((rows, ncols), dtype=bool)
    for r, k in zip(rv, kv):
        m[r, k_map[k]] = True
    cmap = list(k_map) + [1000 + i for i in range(ncols - len(k_map))]  # unmapped columns match nothing
    return O.Table(O.COLMAIN, var, words=bool_to_words(m), mrows=rows, mcols=ncols,
                   col_map=np.asarray(cmap, np.uint32))


@pytest.mark.parametrize("name", sorted(FIXTURE))
def test_reference_unit_test_known_answer(name):
    t = FIXTURE[name]
    expect = t["expect"][-1][1]
    deps = [table(d) for d in t["deps"]]
    if t["operator"] == "HashJoin":
        key, only_count = t["args"][0], t["args"][1] == "true"
        _, _, count = O.hash_join(deps[0], deps[1], var_id(key), only_count)
    else:
        new_var = t["args"][0]
        _, _, count = O.mintersect(deps[0], deps[1:], var_id(new_var), 16, t["args"][2] == "true")
    assert count == expect, (name, t["source"])


def test_fixture_covers_the_reference_tests():
    assert sum(t["operator"] == "HashJoin" for t in FIXTURE.values()) == 8
    assert sum(t["operator"] == "Mintersect" for t in FIXTURE.values()) == 2


def test_restated_vectors_match_the_fixture():
    """The vectors the GPU known-answer tests use (tests/test_oracle_known_answers.py)
    are the reference's, as extracted into the fixture."""
    from tests.test_oracle_known_answers import VA, VK
    for t in FIXTURE.values():
        for d in t["deps"]:
            vals = list(d["vectors"].values())
            assert vals[0] == VA.tolist()
            assert vals[1] == VK.tolist()
