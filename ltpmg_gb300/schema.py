"""Table schemas in the reference's JSON format, mapped onto the column store.

The reference describes its tables in data/*.json: ``{"tables": [{"name",
"size", "attributes": [{"name", "type": "int" | "double" | "string", ...}]}]}``
(parsed by its src/row_parser.cpp).  Here every attribute becomes columns of
a column-store table:

* ``int`` -> one int32 column (the reference's ``int_data``);
* ``double`` -> one int64 column holding a fixed-point value (money as
  cents, as the order-entry workload stores it), or ``double="host"`` to
  leave it with the host program;
* ``string`` -> left with the host program by default (the reference's GPU
  operators never change string fields), or ``string="int32x6"`` for the
  24-byte field as six int32 columns.

``TableSpec.columns`` maps each attribute kept on the device to its first
column and its column count.
"""
import json
from dataclasses import dataclass, field

STRING_COLS = 6  # a 24-byte string field as int32 columns


@dataclass
class TableSpec:
    name: str
    n_cols: int = 0
    wide_cols: int = 0                            # bit c: column c holds int64
    columns: dict = field(default_factory=dict)   # attribute -> (first column, columns)
    host_attributes: list = field(default_factory=list)


def from_reference_json(source, double="int64", string="host"):
    """TableSpecs of a reference schema (a path, a JSON string or the parsed
    dict), in the file's table order."""
    if double not in ("int64", "host") or string not in ("host", "int32x6"):
        raise ValueError("double must be 'int64' or 'host', string 'host' or 'int32x6'")
    if isinstance(source, dict):
        doc = source
    elif isinstance(source, str) and source.lstrip().startswith("{"):
        doc = json.loads(source)
    else:
        with open(source) as f:
            doc = json.load(f)
    specs = []
    for t in doc["tables"]:
        spec = TableSpec(name=t["name"])
        for a in t["attributes"]:
            kind = a["type"]
            if kind == "int":
                width, cols = 4, 1
            elif kind == "double" and double == "int64":
                width, cols = 8, 1
            elif kind == "string" and string == "int32x6":
                width, cols = 4, STRING_COLS
            elif kind in ("double", "string"):
                spec.host_attributes.append(a["name"])
                continue
            else:
                raise ValueError(f"table {t['name']}: unknown attribute type {kind!r}")
            spec.columns[a["name"]] = (spec.n_cols, cols)
            if width == 8:
                spec.wide_cols |= 1 << spec.n_cols
            spec.n_cols += cols
        if spec.n_cols == 0 or spec.n_cols > 64:
            raise ValueError(f"table {t['name']}: {spec.n_cols} device columns (1..64 are possible)")
        specs.append(spec)
    return specs


def create_tables(ctx, specs, rows, rows_cap=None):
    """Creates one table per spec on a Context; rows / rows_cap are an int
    or a {table name: int} map.  Returns {table name: table id}."""
    def pick(v, name, default=None):
        if v is None:
            return default
        return v[name] if isinstance(v, dict) else v

    out = {}
    for s in specs:
        n = pick(rows, s.name)
        wide = [c for c in range(s.n_cols) if (s.wide_cols >> c) & 1]
        out[s.name] = ctx.create_table(n, s.n_cols, rows_cap=pick(rows_cap, s.name, n), wide=wide)
    return out
