// Per-row evaluation of value operands (column, literal or postfix
// arithmetic program) shared by the select and group-by kernels.
#pragma once

#include "common.cuh"

namespace gfpdb {

// ---- dates: days since 1970-01-01 <-> proleptic Gregorian (y, m, d), by the
// era / day-of-era decomposition of Howard Hinnant's public-domain calendar
// algorithms (400-year eras of 146097 days, years starting in March so the
// leap day ends the year).
__host__ __device__ __forceinline__ void civil_from_days(int64_t z, int64_t* y, int* m, int* d) {
  z += 719468;
  const int64_t era = (z >= 0 ? z : z - 146096) / 146097;
  const int64_t doe = z - era * 146097;
  const int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  const int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const int64_t mp = (5 * doy + 2) / 153;
  *d = static_cast<int>(doy - (153 * mp + 2) / 5 + 1);
  *m = static_cast<int>(mp < 10 ? mp + 3 : mp - 9);
  *y = yoe + era * 400 + (*m <= 2 ? 1 : 0);
}

__host__ __device__ __forceinline__ int64_t days_from_civil(int64_t y, int m, int d) {
  y -= m <= 2 ? 1 : 0;
  const int64_t era = (y >= 0 ? y : y - 399) / 400;
  const int64_t yoe = y - era * 400;
  const int64_t doy = (153 * (m > 2 ? m - 3 : m + 9) + 2) / 5 + d - 1;
  const int64_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 719468;
}

__host__ __device__ __forceinline__ int days_in_month(int64_t y, int m) {
  if (m == 2) return ((y % 4 == 0 && y % 100 != 0) || y % 400 == 0) ? 29 : 28;
  return (m == 4 || m == 6 || m == 9 || m == 11) ? 30 : 31;
}

// days plus n days / months / years; a day past the end of the new month
// becomes its last day (Jan 31 + 1 month = Feb 28 or 29).
__host__ __device__ __forceinline__ int64_t date_add(int64_t days, int64_t n, int interval) {
  if (interval == 0) return days + n;
  int64_t y;
  int m, d;
  civil_from_days(days, &y, &m, &d);
  int64_t months = y * 12 + (m - 1) + (interval == 1 ? n : n * 12);
  const int64_t ny = months >= 0 ? months / 12 : -((-months + 11) / 12);
  const int nm = static_cast<int>(months - ny * 12) + 1;
  const int dim = days_in_month(ny, nm);
  return days_from_civil(ny, nm, d < dim ? d : dim);
}

// ---- strings
// SQL LIKE without an escape character: % any run of bytes, _ one byte.
// Greedy, backing up to the last % on a mismatch (linear in the common
// cases, quadratic at worst).
__device__ __forceinline__ bool like_match(const uint8_t* s, int32_t n, const char* pat, int32_t pn) {
  int32_t si = 0, pi = 0, star = -1, mark = 0;
  while (si < n) {
    if (pi < pn && (pat[pi] == '_' || static_cast<uint8_t>(pat[pi]) == s[si])) {
      ++si;
      ++pi;
    } else if (pi < pn && pat[pi] == '%') {
      star = pi++;
      mark = si;
    } else if (star >= 0) {
      pi = star + 1;
      si = ++mark;
    } else {
      return false;
    }
  }
  while (pi < pn && pat[pi] == '%') ++pi;
  return pi == pn;
}

// SUBSTRING(value FROM f FOR n) of bytes [b, e): positions f .. f + n - 1
// (1-based) that fall inside the value.
__device__ __forceinline__ void substring_range(int32_t* b, int32_t* e, int32_t f, int32_t n) {
  const int64_t len = *e - *b;
  int64_t lo = f, hi = static_cast<int64_t>(f) + n;  // [lo, hi) in 1-based positions
  if (lo < 1) lo = 1;
  if (hi > len + 1) hi = len + 1;
  if (hi <= lo) {
    *e = *b;
    return;
  }
  *e = *b + static_cast<int32_t>(hi - 1);
  *b = *b + static_cast<int32_t>(lo - 1);
}

// A utf8 column's value at `row` (or its substring) against a literal of the
// string pool: op LO_STR_EQ / LO_STR_NE / LO_LIKE / LO_NOT_LIKE.
__device__ __forceinline__ bool string_test(int op, const DevCol& c, int64_t row, const char* lit, int32_t lit_len,
                                            bool sub, int32_t sub_from, int32_t sub_len) {
  int32_t b = c.offsets[row], e = c.offsets[row + 1];
  if (sub) substring_range(&b, &e, sub_from, sub_len);
  const uint8_t* bytes = static_cast<const uint8_t*>(c.data) + b;
  const int32_t n = e - b;
  if (op == LO_LIKE || op == LO_NOT_LIKE) return like_match(bytes, n, lit, lit_len) == (op == LO_LIKE);
  bool eq = n == lit_len;
  for (int32_t i = 0; eq && i < n; ++i) eq = bytes[i] == static_cast<uint8_t>(lit[i]);
  return eq == (op == LO_STR_EQ);
}

// Postfix arithmetic for one row (operands that are not a bare column or
// literal). The stack lives in registers/local memory of this thread.
static __device__ __noinline__ int64_t eval_prog(const Program& prog, const DevCol* cols, int begin, int len, int64_t row,
                             DevStatus* st) {
  Scalar stk[kStackDepth];
  int sp = 0;
  for (int pc = begin; pc < begin + len; ++pc) {
    const Instr in = prog.instrs[pc];
    switch (in.op) {
      case IO_COL: {
        const DevCol& c = cols[in.col];
        Scalar s;
        if (c.type == CT_F64) s.i = load_as_i64_bits(c, row);
        else s.i = load_int(c, row);
        stk[sp++] = s;
        break;
      }
      case IO_LIT: stk[sp++] = in.imm; break;
      case IO_ADD:
      case IO_SUB:
      case IO_MUL:
      case IO_DIV: {
        Scalar b = stk[--sp];
        Scalar a = stk[sp - 1];
        Scalar r;
        if (in.vt == VT_F64) {
          switch (in.op) {
            case IO_ADD: r.f = a.f + b.f; break;
            case IO_SUB: r.f = a.f - b.f; break;
            case IO_MUL: r.f = a.f * b.f; break;
            default: r.f = a.f / b.f; break;
          }
        } else {
          const uint64_t ua = static_cast<uint64_t>(a.i), ub = static_cast<uint64_t>(b.i);
          switch (in.op) {
            case IO_ADD: r.i = static_cast<int64_t>(ua + ub); break;  // two's-complement wrap
            case IO_SUB: r.i = static_cast<int64_t>(ua - ub); break;
            case IO_MUL: r.i = static_cast<int64_t>(ua * ub); break;
            default:
              if (b.i == 0) {
                raise_status(st, GFPDB_EDEVICE, 2);  // integer divide by zero
                r.i = 0;
              } else if (a.i == INT64_MIN && b.i == -1) {
                r.i = INT64_MIN;
              } else {
                r.i = a.i / b.i;
              }
          }
        }
        stk[sp - 1] = r;
        break;
      }
      case IO_NEG:
        if (in.vt == VT_F64) stk[sp - 1].f = -stk[sp - 1].f;
        else stk[sp - 1].i = static_cast<int64_t>(0ull - static_cast<uint64_t>(stk[sp - 1].i));
        break;
      case IO_I2F: stk[sp - 1].f = static_cast<double>(stk[sp - 1].i); break;
      case IO_F2I: stk[sp - 1].i = static_cast<int64_t>(stk[sp - 1].f); break;
      case IO_WRAP32: stk[sp - 1].i = static_cast<int32_t>(static_cast<uint32_t>(stk[sp - 1].i)); break;
      case IO_EXTRACT: {
        int64_t y;
        int m, d;
        civil_from_days(stk[sp - 1].i, &y, &m, &d);
        stk[sp - 1].i = in.imm.i == 0 ? d : (in.imm.i == 1 ? m : y);
        break;
      }
      case IO_DATE_ADD: {
        const int64_t n = stk[--sp].i;
        stk[sp - 1].i = date_add(stk[sp - 1].i, n, static_cast<int>(in.imm.i));
        break;
      }
      case IO_CMP: {
        const Scalar b = stk[--sp];
        const Scalar a = stk[sp - 1];
        bool r;
        if (in.vt == VT_F64) {
          switch (in.imm.i) {
            case LO_LT: r = a.f < b.f; break;
            case LO_LE: r = a.f <= b.f; break;
            case LO_GT: r = a.f > b.f; break;
            case LO_GE: r = a.f >= b.f; break;
            case LO_EQ: r = a.f == b.f; break;
            default: r = a.f != b.f; break;
          }
        } else {
          switch (in.imm.i) {
            case LO_LT: r = a.i < b.i; break;
            case LO_LE: r = a.i <= b.i; break;
            case LO_GT: r = a.i > b.i; break;
            case LO_GE: r = a.i >= b.i; break;
            case LO_EQ: r = a.i == b.i; break;
            default: r = a.i != b.i; break;
          }
        }
        stk[sp - 1].i = r ? 1 : 0;
        break;
      }
      case IO_AND: {
        const int64_t b = stk[--sp].i;
        stk[sp - 1].i = (stk[sp - 1].i != 0 && b != 0) ? 1 : 0;
        break;
      }
      case IO_OR: {
        const int64_t b = stk[--sp].i;
        stk[sp - 1].i = (stk[sp - 1].i != 0 || b != 0) ? 1 : 0;
        break;
      }
      case IO_NOT: stk[sp - 1].i = stk[sp - 1].i != 0 ? 0 : 1; break;
      case IO_SELECT: {
        const Scalar e = stk[--sp];
        const Scalar t = stk[--sp];
        stk[sp - 1] = stk[sp - 1].i != 0 ? t : e;
        break;
      }
      case IO_STR_TEST: {
        const int64_t k = in.imm.i;
        const bool sub = (k >> 40) & 1;
        const bool r = string_test(static_cast<int>(k & 0xff), cols[in.col], row,
                                   prog.strpool + ((k >> 8) & 0xffff), static_cast<int32_t>((k >> 24) & 0xffff), sub,
                                   static_cast<int16_t>(static_cast<uint32_t>(in.pad) >> 16),
                                   static_cast<int32_t>(static_cast<uint32_t>(in.pad) & 0xffff));
        Scalar s;
        s.i = r ? 1 : 0;
        stk[sp++] = s;
        break;
      }
      default: break;
    }
  }
  return stk[0].i;
}

// Value of an operand for one row, as int64 bits (doubles bit-cast).
__device__ __forceinline__ int64_t operand_row(const Program& prog, const DevCol* cols, const Operand& o, int64_t row,
                                               DevStatus* st) {
  if (o.kind == OPND_COL) {
    const DevCol& c = cols[o.col];
    return c.type == CT_F64 ? load_as_i64_bits(c, row) : load_int(c, row);
  }
  if (o.kind == OPND_LIT) return o.lit.i;
  return eval_prog(prog, cols, o.prog_begin, o.prog_len, row, st);
}

}  // namespace gfpdb
