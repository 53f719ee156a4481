"""Write the Parquet fixtures of tests/golden/parquet/ with pyarrow (run
here, where pyarrow is installed; the GPU tests only read the files):
the seeded tables of parquet_source.py under several writer settings (plain
and dictionary encodings, no compression and snappy, data pages v1 and v2,
several row groups and many small pages, optional and required columns),
plus files the reader must refuse (nulls, gzip, a boolean column). Also
writes layout.json: each file's row groups (first column chunk's offset and
rows) for the range-read test.

    python tests/golden/make_parquet.py
"""

import json
import sys
from pathlib import Path

import numpy as np
import pyarrow as pa
import pyarrow.parquet as pq

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from parquet_source import FIXTURES, source  # noqa: E402

OUT = HERE / "parquet"
TYPES = {"int32": pa.int32(), "int64": pa.int64(), "float64": pa.float64(), "date32": pa.date32(), "utf8": pa.string()}


def table(n, seed, required):
    cols = source(n, seed)
    fields, arrays = [], []
    for name, (ty, vals) in cols.items():
        fields.append(pa.field(name, TYPES[ty], nullable=not required))
        arrays.append(pa.array(vals, type=TYPES[ty]))
    return pa.Table.from_arrays(arrays, schema=pa.schema(fields))


def main():
    OUT.mkdir(exist_ok=True)
    layout = {}
    for name, (n, seed, opts, required) in FIXTURES.items():
        path = OUT / f"{name}.parquet"
        t = table(n, seed, required)
        pq.write_table(t, path, **opts)
        back = pq.read_table(path)
        assert back.equals(t), name
        md = pq.ParquetFile(path).metadata
        groups = []
        for g in range(md.num_row_groups):
            c0 = md.row_group(g).column(0)
            off = c0.dictionary_page_offset if c0.has_dictionary_page else c0.data_page_offset
            groups.append({"offset": off, "rows": md.row_group(g).num_rows})
        layout[name] = groups
    # files the reader refuses
    rng = np.random.default_rng(3)
    vals = pa.array([None if i % 7 == 0 else int(v) for i, v in enumerate(rng.integers(0, 100, 500))], pa.int64())
    pq.write_table(pa.table({"x": vals}), OUT / "nulls.parquet")
    pq.write_table(pa.table({"x": pa.array(np.arange(500, dtype=np.int64))}), OUT / "gzip.parquet", compression="GZIP")
    pq.write_table(pa.table({"x": pa.array(np.arange(500, dtype=np.int64)), "b": pa.array(np.arange(500) % 2 == 0)}),
                   OUT / "bools.parquet")
    (OUT / "layout.json").write_text(json.dumps(layout, indent=1) + "\n")


if __name__ == "__main__":
    main()
