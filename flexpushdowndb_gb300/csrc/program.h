// Device-side program and parameter structures shared by the host compiler
// (host/expr.cpp) and the kernels. Plain structs only: they are copied into
// kernel parameter space, so every field is read through the constant bank
// and is uniform across a warp.
//
// A predicate is lowered to conjunctive normal form: the row is selected when
// every clause holds, and a clause holds when any of its leaves holds. A leaf
// compares two operands (column, literal, or a short postfix arithmetic
// program); NOT is pushed into the leaves by negating their comparison, which
// also gives SQL's "a NULL predicate does not select the row" rule that
// Gandiva filters follow (fpdb-expression-gandiva/src/Filter.cpp:178-225).
#pragma once

#include <stdint.h>

namespace gfpdb {

enum ColTypeCode : int8_t { CT_I32 = 0, CT_I64 = 1, CT_DATE32 = 2, CT_F64 = 3, CT_UTF8 = 4 };
enum ValType : int8_t { VT_I64 = 0, VT_F64 = 1 };

constexpr int kMaxCols = 24;
constexpr int kMaxLeaves = 32;
constexpr int kMaxClauses = 16;
constexpr int kMaxInstrs = 48;
constexpr int kMaxBlooms = 8;
constexpr int kStackDepth = 8;
constexpr int kMaxAggs = 8;

struct DevCol {
  const void* data;        // values (utf8: bytes)
  const int32_t* offsets;  // utf8 only
  int32_t type;            // ColTypeCode
  int32_t pad;
};

union Scalar {
  int64_t i;
  double f;
};

enum OperandKind : int8_t { OPND_COL = 0, OPND_LIT = 1, OPND_PROG = 2 };

struct Operand {
  int8_t kind;  // OperandKind
  int8_t vt;    // ValType of the operand's value
  int16_t col;  // OPND_COL: column slot
  int16_t prog_begin;
  int16_t prog_len;  // OPND_PROG: instrs[prog_begin, prog_begin + prog_len)
  Scalar lit;        // OPND_LIT
};

enum LeafOp : int8_t {
  LO_LT = 0, LO_LE, LO_GT, LO_GE, LO_EQ, LO_NE,
  LO_TRUE, LO_FALSE,
  LO_STR_EQ, LO_STR_NE,     // utf8 column vs utf8 literal held in the string pool
  LO_STRCOL_EQ, LO_STRCOL_NE, // utf8 column vs utf8 column (lhs.col, rhs.col)
  LO_LIKE, LO_NOT_LIKE        // utf8 column matched against a LIKE pattern held in the string pool
};
// LO_STR_EQ / NE and LO_LIKE / NOT_LIKE may test a substring of the column
// (SUBSTRING(col FROM f FOR n) = 'x'): then rhs.col is 1, rhs.prog_begin the
// first position f (1-based, may be <= 0) and rhs.prog_len the length n; an
// all-zero rhs tests the whole value.

struct Leaf {
  int8_t op;      // LeafOp
  int8_t cmp_vt;  // comparison done in int64 or double
  int16_t str_begin;  // LO_STR_*: literal bytes in Program::strpool
  int16_t str_len;
  int16_t pad;
  Operand lhs;
  Operand rhs;
};

enum InstrOp : int8_t {
  IO_COL = 0,  // push column value (as int64 or double per vt)
  IO_LIT,      // push immediate
  IO_ADD, IO_SUB, IO_MUL, IO_DIV,  // pop b, pop a, push a op b (vt = result type)
  IO_NEG,
  IO_I2F,      // int64 -> double
  IO_F2I,      // double -> int64 (truncation, as castBIGINT)
  IO_WRAP32,   // keep the low 32 bits and sign-extend (int32 arithmetic results)
  IO_EXTRACT,  // date32 days -> the day (imm 0), month (1) or year (2) of the date
  IO_DATE_ADD, // pop n, pop days: days plus n days (imm 0), months (1) or years (2)
  IO_CMP,      // pop b, pop a: 1 if a <op> b else 0 (imm = LeafOp LO_LT..LO_NE, vt = comparison type)
  IO_AND, IO_OR,  // pop b, pop a: a and / or b (0 / 1)
  IO_NOT,      // 1 - a
  IO_SELECT,   // pop else, pop then, pop cond: cond ? then : else
  IO_STR_TEST  // push 0 / 1: utf8 column `col` against the string pool (the leaf test of
               // imm.i & 0xff = LeafOp LO_STR_EQ / NE / LIKE / NOT_LIKE, pool range
               // (imm.i >> 8) & 0xffff, length (imm.i >> 24) & 0xffff; bit 40 of imm.i set:
               // a substring, first position (int16) pad >> 16, length pad & 0xffff)
};

struct Instr {
  int8_t op;
  int8_t vt;
  int16_t col;
  int32_t pad;
  Scalar imm;
};

constexpr int kStrPool = 128;

struct Program {
  int32_t n_leaves;
  int32_t n_clauses;   // 0 = always true
  int32_t n_instrs;
  int32_t pad;
  int16_t clause_begin[kMaxClauses + 1];  // leaves[clause_begin[c], clause_begin[c+1])
  Leaf leaves[kMaxLeaves];
  Instr instrs[kMaxInstrs];
  char strpool[kStrPool];
};

// Aggregate input: an operand evaluated per row (count(*) has kind OPND_LIT).
enum AggFn : int8_t {
  AGG_SUM = 0, AGG_COUNT = 1, AGG_MIN = 2, AGG_MAX = 3, AGG_COUNT_STAR = 4, AGG_AVG = 5,
  AGG_AVG_REDUCE = 6  // second phase of a parallel AVG: sum of partial sums / sum of partial counts
};

struct AggSpec {
  int8_t fn;  // AggFn
  int8_t vt;  // value type of the input (sum of doubles is an f64 sum)
  int16_t pad;
  int32_t pad2;
  Operand in;
};

}  // namespace gfpdb
