"""Tables described in the reference's JSON schema format (data/*.json)
mapped onto the column store (ltpmg_gb300/schema.py): CPU checks of the
mapping, and on the GPU a table created from a schema runs a batch against
the oracle."""
import json

import numpy as np
import pytest

from ltpmg_gb300 import schema as S

# the reference's schema layout: tables of typed attributes
DOC = {"tables": [
    {"name": "accounts", "size": 4, "attributes": [
        {"name": "id", "type": "int", "data_distribution": "dist"},
        {"name": "owner", "type": "string", "data_distribution": "dist"},
        {"name": "balance", "type": "double", "data_distribution": "dist"},
        {"name": "visits", "type": "int", "data_distribution": "dist"}]},
    {"name": "events", "size": 4, "attributes": [
        {"name": "kind", "type": "int", "data_distribution": "dist"}]},
]}


def test_default_mapping_keeps_strings_on_the_host():
    a, e = S.from_reference_json(DOC)
    assert (a.name, a.n_cols, a.wide_cols) == ("accounts", 3, 0b010)
    assert a.columns == {"id": (0, 1), "balance": (1, 1), "visits": (2, 1)}
    assert a.host_attributes == ["owner"]
    assert (e.n_cols, e.columns) == (1, {"kind": (0, 1)})


def test_strings_as_int32_columns_and_doubles_on_the_host(tmp_path):
    p = tmp_path / "schema.json"
    p.write_text(json.dumps(DOC))
    a, _ = S.from_reference_json(str(p), double="host", string="int32x6")
    assert a.columns == {"id": (0, 1), "owner": (1, 6), "visits": (7, 1)}
    assert (a.n_cols, a.wide_cols, a.host_attributes) == (8, 0, ["balance"])
    assert S.from_reference_json(json.dumps(DOC))[0].n_cols == 3


def test_rejects_unknown_types_and_empty_tables():
    with pytest.raises(ValueError):
        S.from_reference_json({"tables": [{"name": "x", "attributes": [{"name": "y", "type": "blob"}]}]})
    with pytest.raises(ValueError):
        S.from_reference_json({"tables": [{"name": "x", "attributes": [{"name": "y", "type": "string"}]}]})


@pytest.mark.gpu
def test_tables_from_a_schema_run_a_batch():
    import ltpmg_gb300 as G
    import oracle as O

    specs = S.from_reference_json(DOC)
    with G.Context(device=0) as ctx:
        ids = S.create_tables(ctx, specs, rows={"accounts": 1000, "events": 10})
        t = ids["accounts"]
        init = np.arange(3000, dtype=np.int64).reshape(3, 1000) * 7
        for c in range(3):
            ctx.upload_column(t, c, init[c].astype(np.int64 if c == 1 else np.int32))
        # RMW on balance (int64) and visits (int32), reads of id
        tf = np.array([0, 3, 5], np.uint32)
        keys = np.array([5, 5, 9, 5, 9], np.uint64)
        opw = np.array([O.opword(1, 1, t, 250), O.opword(1, 2, t, 1), O.opword(0, 0, t, 0),
                        O.opword(1, 1, t, -50), O.opword(0, 2, t, 0)], np.uint32)
        b = ctx.batch(2, 5)
        b.load(tf, keys, opw)
        b.execute()
        commit, vals, st = b.results64()
        assert commit.tolist() == [1, 1]
        assert vals.tolist() == [init[1, 5] + 250, init[2, 5] + 1, init[0, 9], init[1, 5] + 200, init[2, 9]]
