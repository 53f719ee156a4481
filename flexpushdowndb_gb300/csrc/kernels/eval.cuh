// Per-row evaluation of value operands (column, literal or postfix
// arithmetic program) shared by the select and group-by kernels.
#pragma once

#include "common.cuh"

namespace gfpdb {

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
