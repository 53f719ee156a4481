"""Pin the oracle to the reference's own known-answer tests.

Each case restates, in this project's vocabulary, the inputs and expected
values of a reference test (cited per test); the oracle must reproduce them.
The same cases run on the GPU path in test_pins_gpu.py.
"""

import numpy as np
import pytest

from flexpushdowndb_gb300.expression import cast, col, lt, num_lit, times
from flexpushdowndb_gb300.tupleset import Column, Table
from oracle import expr as oexpr
from oracle import ops as oops

# fpdb-expression-gandiva/test/TestUtil.h:25-45: columns a, b, c = "1".."3", "4".."6", "7".."9"
ABC_CSV = b"1,4,7\n2,5,8\n3,6,9\n"
ABC_FIELDS = [("a", "int64"), ("b", "int64"), ("c", "int64")]


def abc_table():
    return oops.csv_parse(ABC_CSV, ABC_FIELDS)


def test_multiply_known_products():
    # fpdb-expression-gandiva/test/MultiplyTest.cpp:35-52: a*b as float64 = 4, 10, 18
    t = abc_table()
    v, ty = oexpr.value(times(cast(col("a"), "float64"), cast(col("b"), "float64")), t)
    assert ty == "float64"
    assert v.tolist() == [4.0, 10.0, 18.0]


def test_less_than_truth_table():
    # fpdb-expression-gandiva/test/BinaryExpressionTest.cpp:35-57
    t = abc_table()
    for name, k in (("a", 2), ("b", 5), ("c", 8)):
        m = oexpr.predicate(lt(cast(col(name), "int32"), num_lit(k, "int32")), t)
        assert m.tolist() == [True, False, False]


@pytest.mark.parametrize("ty", ["int32", "int64", "float64"])
def test_cast_values(ty):
    # fpdb-expression-gandiva/test/CastTest.cpp:81-137: a[0]=1, b[1]=5, c[2]=9
    t = abc_table()
    assert oexpr.value(cast(col("a"), ty), t)[0][0] == 1
    assert oexpr.value(cast(col("b"), ty), t)[0][1] == 5
    assert oexpr.value(cast(col("c"), ty), t)[0][2] == 9


def test_csv_test_file():
    # fpdb-tuple/data/csv/test.csv as fpdb-tuple/test/CSVTest.cpp:35-79,192 describes it:
    # header A,B,C then rows 1,2,3 / 4,5,6 / 7,8,9; 24 bytes.
    text = b"A,B,C\n1,2,3\n4,5,6\n7,8,9\n"
    assert len(text) == 24
    t = oops.csv_parse(text, [("a", "utf8"), ("b", "utf8"), ("c", "utf8")], has_header=True)
    assert t.rows() == [("1", "2", "3"), ("4", "5", "6"), ("7", "8", "9")]
    t2 = oops.csv_parse(text, [("a", "utf8"), ("b", "utf8"), ("c", "utf8")], columns=["a", "b"], has_header=True)
    assert t2.names == ["a", "b"] and t2.num_rows == 3


def csv_3x10000() -> bytes:
    # fpdb-tuple/data/csv/test3x10000.csv per CSVTest.cpp:203 and
    # FileReaderTestUtil::checkReadWholeAllTestCsv3x10000: header, then 10000
    # rows cycling 1,2,3 / 4,5,6 / 7,8,9; 60006 bytes.
    rows = [b"1,2,3\n", b"4,5,6\n", b"7,8,9\n"]
    return b"A,B,C\n" + b"".join(rows[r % 3] for r in range(10000))


def test_csv_3x10000():
    text = csv_3x10000()
    assert len(text) == 60006
    t = oops.csv_parse(text, [("a", "int32"), ("b", "int32"), ("c", "int32")], has_header=True)
    assert t.num_rows == 10000
    a = t["a"]
    assert a[0] == 1 and a[1] == 4 and a[2] == 7 and a[9999] == 1


# fpdb-executor/ATTIC/test/data/group/a.csv and .../join/{a,b}.csv
GROUP_A = b"aa,ab,ac\n10,13,16\n10,14,17\n12,15,18\n"
JOIN_B = b"ba,bb,bc\n10,23,26\n11,24,27\n10,25,28\n"


def test_attic_group_sum():
    # fpdb-executor/ATTIC/test/GroupTest.cpp:137-150: group by AA, sum(AB) -> 10: 27, 12: 15
    t = oops.csv_parse(GROUP_A, [("aa", "int64"), ("ab", "int64"), ("ac", "int64")], has_header=True)
    g = oops.group_by(t, ["aa"], [{"function": "SUM", "name": "sum", "expr": col("ab")}])
    assert g.sorted_rows() == [(10, 27), (12, 15)]


def test_attic_join():
    # fpdb-executor/ATTIC/test/JoinTest.cpp:82-123: a join b on aa = ba -> 4 rows
    a = oops.csv_parse(GROUP_A, [("aa", "int64"), ("ab", "int64"), ("ac", "int64")], has_header=True)
    b = oops.csv_parse(JOIN_B, [("ba", "int64"), ("bb", "int64"), ("bc", "int64")], has_header=True)
    j = oops.hash_join(b, a, "ba", "aa")  # probe a, build b: output a's columns then b's
    assert j.names == ["aa", "ab", "ac", "ba", "bb", "bc"]
    assert j.sorted_rows() == sorted([
        (10, 13, 16, 10, 23, 26), (10, 13, 16, 10, 25, 28), (10, 14, 17, 10, 23, 26), (10, 14, 17, 10, 25, 28)])


def test_int32_multiply_wraps():
    # Gandiva's multiply(int32, int32) returns int32 (same-type operands keep
    # their type, BinaryExpression.cpp:57-102), so products wrap.
    t = Table([Column("x", "int32", [70000, -3]), Column("y", "int32", [70000, 5])])
    v, ty = oexpr.value(times(col("x"), col("y")), t)
    assert ty == "int32"
    assert v.tolist() == [np.int32(np.int64(70000 * 70000) - 2**32), -15]


def test_bloom_no_false_negatives_and_fpr():
    rng = np.random.default_rng(7)
    keys = rng.choice(10**7, size=20000, replace=False)
    w = oops.bloom_words(keys, 10, 3)
    assert oops.bloom_contains(w, keys, 3).all()
    others = np.setdiff1d(rng.choice(10**7, size=200000, replace=False), keys)
    fpr = oops.bloom_contains(w, others, 3).mean()
    # k=3, 10 bits/key: about 1.7% for a flat filter; blocking adds a little
    assert fpr < 0.035
