"""CPU oracle: a restatement of the reference's operator semantics.

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs may import or run anything in this directory;
the library never does, and it is never the thing measured or shipped.

Contents:
  expr.py   - expression evaluation with the reference's typing rules
  ops.py    - filter, blocked bloom, inner hash join, hash group-by, CSV
  queries.py- the two-table and star queries composed from ops.py
  baseline.c- multi-threaded C restatement of the star / two-table queries,
              timed as the CPU baseline (built by the Makefile here)

Parity pins: the expression and CSV rules are checked against the known
answers of the reference's own tests (restated in tests/test_oracle_pins.py)
and the join / group / filter paths against pyarrow's acero (the successor
of the Arrow 6 engine the reference calls) through the committed fixtures in
tests/golden/ (generated by tests/golden/make_golden.py).
"""
