"""The seeded tables the Parquet fixtures hold (TEST INFRASTRUCTURE ONLY):
make_parquet.py writes them with pyarrow, and the GPU tests regenerate the
same values here to compare the device reader's output with, so no decoder
stands between the written values and the check."""

from __future__ import annotations

import numpy as np

WORDS = ["", "a", "ab", "MEDIUM BRUSHED STEEL", "PROMO ANODIZED TIN", "x" * 40, "naïve café", "中文字符",
         "STANDARD", "ECONOMY POLISHED COPPER"]


def source(n: int, seed: int) -> dict:
    """name -> (arrow type name, values): int32, int64, float64, date32
    and utf8 columns, some with few distinct values (dictionary pages),
    some all distinct."""
    rng = np.random.default_rng(seed)
    return {
        "i32": ("int32", rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)),
        "i64": ("int64", rng.integers(-2**62, 2**62, n, dtype=np.int64)),
        "f64": ("float64", rng.normal(0.0, 1e6, n)),
        "d": ("date32", rng.integers(-30000, 30000, n).astype(np.int32)),
        "k": ("int64", rng.integers(0, 20, n).astype(np.int64) * 1_000_003),
        "s": ("utf8", [WORDS[i] for i in rng.integers(0, len(WORDS), n)]),
        "u": ("utf8", [f"row-{i}-{v}" for i, v in enumerate(rng.integers(0, 10**9, n).tolist())]),
    }


FIXTURES = {
    # file: (rows, seed, pyarrow write options, columns are REQUIRED)
    "plain_none_v1": (8000, 11, dict(use_dictionary=False, compression="NONE", data_page_version="1.0",
                                     row_group_size=3000, data_page_size=4096), False),
    "dict_snappy_v1": (8000, 12, dict(use_dictionary=True, compression="SNAPPY", data_page_version="1.0",
                                      row_group_size=3000, data_page_size=4096), False),
    "dict_snappy_v2": (8000, 13, dict(use_dictionary=True, compression="SNAPPY", data_page_version="2.0",
                                      row_group_size=2500, data_page_size=4096), False),
    "plain_snappy_v2": (8000, 14, dict(use_dictionary=False, compression="SNAPPY", data_page_version="2.0",
                                       row_group_size=8000, data_page_size=8192), False),
    "required_dict_none": (5000, 15, dict(use_dictionary=True, compression="NONE", data_page_version="1.0",
                                          row_group_size=5000), True),
    "one_row": (1, 16, dict(compression="SNAPPY"), False),
}
