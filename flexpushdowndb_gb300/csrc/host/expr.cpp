#include "expr.h"

#include <algorithm>
#include <cstring>
#include <sstream>

namespace gfpdb {

namespace {

bool is_int_type(DType t) { return t == DType::Int32 || t == DType::Int64 || t == DType::Date32; }

DType literal_type_from_name(const std::string& n, bool* is_bool) {
  *is_bool = false;
  if (n == "boolean" || n == "Boolean" || n == "bool") {
    *is_bool = true;
    return DType::Int32;
  }
  return dtype_from_name(n);
}

LeafOp negate(LeafOp op) {
  switch (op) {
    case LO_LT: return LO_GE;
    case LO_LE: return LO_GT;
    case LO_GT: return LO_LE;
    case LO_GE: return LO_LT;
    case LO_EQ: return LO_NE;
    case LO_NE: return LO_EQ;
    case LO_TRUE: return LO_FALSE;
    case LO_FALSE: return LO_TRUE;
    case LO_STR_EQ: return LO_STR_NE;
    case LO_STR_NE: return LO_STR_EQ;
    case LO_STRCOL_EQ: return LO_STRCOL_NE;
    case LO_STRCOL_NE: return LO_STRCOL_EQ;
    case LO_LIKE: return LO_NOT_LIKE;
    case LO_NOT_LIKE: return LO_LIKE;
  }
  return op;
}

const char* cmp_name(LeafOp op) {
  switch (op) {
    case LO_LT: return "<";
    case LO_LE: return "<=";
    case LO_GT: return ">";
    case LO_GE: return ">=";
    case LO_EQ: return "=";
    case LO_NE: return "!=";
    default: return "?";
  }
}

const char* arith_name(InstrOp op) {
  switch (op) {
    case IO_ADD: return "+";
    case IO_SUB: return "-";
    case IO_MUL: return "*";
    case IO_DIV: return "/";
    default: return "?";
  }
}

Scalar parse_scalar(const json::Value& v, DType t, bool is_bool) {
  Scalar s{};
  if (is_bool) {
    s.i = v.kind == json::Value::Bool ? (v.b ? 1 : 0) : (v.integer() != 0);
  } else if (t == DType::Float64) {
    s.f = v.number();
  } else {
    if (v.kind == json::Value::Number && !v.is_integer) fail(GFPDB_EINVAL, "integer literal expected");
    s.i = v.integer();
    if (t == DType::Int32 || t == DType::Date32) s.i = static_cast<int32_t>(s.i);
  }
  return s;
}

std::shared_ptr<Expr> node(Expr::Kind k) {
  auto e = std::make_shared<Expr>();
  e->kind = k;
  return e;
}

}  // namespace

ExprPtr parse_expr(const json::Value& v) {
  const std::string type = v.at("type").str();
  auto binary = [&](Expr::Kind k) {
    auto e = node(k);
    e->kids.push_back(parse_expr(v.at("left")));
    e->kids.push_back(parse_expr(v.at("right")));
    return e;
  };
  if (type == "Column") {
    auto e = node(Expr::Column);
    e->name = v.contains("columnName") ? v.at("columnName").str() : v.at("name").str();
    return e;
  }
  if (type == "NumericLiteral" || type.rfind("NumericLiteral<", 0) == 0) {
    auto e = node(Expr::Literal);
    std::string dt = v.get_str("dataType", "");
    if (dt.empty() && type.size() > 15) dt = type.substr(15, type.size() - 16);
    e->type = literal_type_from_name(dt, &e->is_bool);
    if (v.contains("value") && v.at("value").kind != json::Value::Null)
      e->lit = parse_scalar(v.at("value"), e->type, e->is_bool);
    else
      e->lit_null = true;
    return e;
  }
  if (type == "StringLiteral") {
    auto e = node(Expr::StrLiteral);
    if (v.contains("value")) e->str = v.at("value").str();
    else e->lit_null = true;
    return e;
  }
  if (type == "And" || type == "Or") {
    auto e = node(type == "And" ? Expr::And : Expr::Or);
    if (v.contains("exprs")) {
      for (auto& k : v.at("exprs").array()) e->kids.push_back(parse_expr(k));
    } else {
      e->kids.push_back(parse_expr(v.at("left")));
      e->kids.push_back(parse_expr(v.at("right")));
    }
    if (e->kids.empty()) fail(GFPDB_EINVAL, type + " without operands");
    return e;
  }
  if (type == "Not" || type == "IsNull") {
    auto e = node(type == "Not" ? Expr::Not : Expr::IsNull);
    e->kids.push_back(parse_expr(v.at("expr")));
    return e;
  }
  if (type == "Cast") {
    auto e = node(Expr::Cast);
    e->kids.push_back(parse_expr(v.at("expr")));
    bool b = false;
    e->type = literal_type_from_name(v.at("dataType").str(), &b);
    if (b) fail(GFPDB_EUNSUPPORTED, "cast to boolean");
    return e;
  }
  if (type == "In") {
    auto e = node(Expr::In);
    e->kids.push_back(parse_expr(v.at("expr")));
    bool b = false;
    e->type = literal_type_from_name(v.get_str("dataType", "int64"), &b);
    for (auto& x : v.at("values").array()) {
      if (e->type == DType::Utf8) e->in_strs.push_back(x.str());
      else e->in_values.push_back(parse_scalar(x, e->type, false));
    }
    return e;
  }
  struct { const char* n; LeafOp op; } cmps[] = {
      {"EqualTo", LO_EQ}, {"NotEqualTo", LO_NE}, {"LessThan", LO_LT}, {"LessThanOrEqualTo", LO_LE},
      {"GreaterThan", LO_GT}, {"GreaterThanOrEqualTo", LO_GE}};
  for (auto& c : cmps) {
    if (type == c.n) {
      auto e = binary(Expr::Compare);
      e->cmp = c.op;
      return e;
    }
  }
  struct { const char* n; InstrOp op; } ariths[] = {
      {"Add", IO_ADD}, {"Subtract", IO_SUB}, {"Multiply", IO_MUL}, {"Divide", IO_DIV}};
  for (auto& a : ariths) {
    if (type == a.n) {
      auto e = binary(Expr::Arith);
      e->arith = a.op;
      return e;
    }
  }
  // DateIntervalType names (fpdb-expression-gandiva/src/DateIntervalType.cpp:11-33)
  auto interval = [&](const std::string& s) {
    if (s == "Day") return 0;
    if (s == "Month") return 1;
    if (s == "Year") return 2;
    fail(GFPDB_EINVAL, "unsupported date interval type: '" + s + "'");
  };
  if (type == "DateExtract") {  // DateExtract.cpp:45-63: {"dateExpr", "intervalType"}
    auto e = node(Expr::DateExtract);
    e->kids.push_back(parse_expr(v.at("dateExpr")));
    e->interval = interval(v.at("intervalType").str());
    return e;
  }
  if (type == "DateAdd") {  // DateAdd.cpp: {"left", "right", "intervalType"}
    auto e = binary(Expr::DateAdd);
    e->interval = interval(v.at("intervalType").str());
    return e;
  }
  if (type == "If") {  // If.cpp:49-88: {"ifExpr", "thenExpr", "elseExpr"}
    auto e = node(Expr::If);
    e->kids = {parse_expr(v.at("ifExpr")), parse_expr(v.at("thenExpr")), parse_expr(v.at("elseExpr"))};
    return e;
  }
  if (type == "Like") return binary(Expr::Like);  // Like.cpp: {"left", "right"}
  if (type == "Substr") {  // Substr.cpp:48-88: {"expr", "fromLit", "forLit"}
    auto e = node(Expr::Substr);
    e->kids = {parse_expr(v.at("expr")), parse_expr(v.at("fromLit")), parse_expr(v.at("forLit"))};
    return e;
  }
  fail(GFPDB_EINVAL, "unsupported expression type: '" + type + "'");
}

ExprPtr parse_expr_json(const std::string& text) {
  try {
    return parse_expr(json::parse(text));
  } catch (const Error&) {
    throw;
  } catch (const std::exception& ex) {
    fail(GFPDB_EINVAL, ex.what());
  }
}

std::string expr_to_string(const ExprPtr& e) {
  std::ostringstream os;
  switch (e->kind) {
    case Expr::Column: os << e->name; break;
    case Expr::Literal:
      if (e->lit_null) os << "null";
      else if (e->is_bool) os << (e->lit.i ? "true" : "false");
      else if (e->type == DType::Float64) os << e->lit.f;
      else os << e->lit.i;
      break;
    case Expr::StrLiteral: os << "'" << e->str << "'"; break;
    case Expr::And:
    case Expr::Or: {
      os << "(";
      for (size_t i = 0; i < e->kids.size(); ++i) {
        if (i) os << (e->kind == Expr::And ? " and " : " or ");
        os << expr_to_string(e->kids[i]);
      }
      os << ")";
      break;
    }
    case Expr::Not: os << "not(" << expr_to_string(e->kids[0]) << ")"; break;
    case Expr::IsNull: os << "isnull(" << expr_to_string(e->kids[0]) << ")"; break;
    case Expr::Compare:
      os << "(" << expr_to_string(e->kids[0]) << " " << cmp_name(e->cmp) << " " << expr_to_string(e->kids[1]) << ")";
      break;
    case Expr::Arith:
      os << "(" << expr_to_string(e->kids[0]) << " " << arith_name(e->arith) << " " << expr_to_string(e->kids[1])
         << ")";
      break;
    case Expr::Cast: os << "cast(" << expr_to_string(e->kids[0]) << " as " << dtype_name(e->type) << ")"; break;
    case Expr::In: os << "in(" << expr_to_string(e->kids[0]) << ", " << (e->in_values.size() + e->in_strs.size()) << " values)"; break;
    case Expr::DateExtract:
      os << "extract" << (e->interval == 0 ? "Day" : e->interval == 1 ? "Month" : "Year") << "("
         << expr_to_string(e->kids[0]) << ")";
      break;
    case Expr::DateAdd:
      os << "dateadd" << (e->interval == 0 ? "Day" : e->interval == 1 ? "Month" : "Year") << "("
         << expr_to_string(e->kids[0]) << ", " << expr_to_string(e->kids[1]) << ")";
      break;
    case Expr::If:
      os << "if(" << expr_to_string(e->kids[0]) << ", " << expr_to_string(e->kids[1]) << ", "
         << expr_to_string(e->kids[2]) << ")";
      break;
    case Expr::Like: os << "(" << expr_to_string(e->kids[0]) << " like " << expr_to_string(e->kids[1]) << ")"; break;
    case Expr::Substr:
      os << "substr(" << expr_to_string(e->kids[0]) << ", " << expr_to_string(e->kids[1]) << ", "
         << expr_to_string(e->kids[2]) << ")";
      break;
  }
  return os.str();
}

void expr_columns(const ExprPtr& e, std::vector<std::string>& out) {
  if (e->kind == Expr::Column) {
    if (std::find(out.begin(), out.end(), e->name) == out.end()) out.push_back(e->name);
    return;
  }
  for (auto& k : e->kids) expr_columns(k, out);
}

int ColumnSlots::slot_for(const std::string& name, DType t) {
  for (size_t i = 0; i < names.size(); ++i)
    if (names[i] == name) return static_cast<int>(i);
  if (static_cast<int>(names.size()) >= kMaxCols) fail(GFPDB_EUNSUPPORTED, "expression references too many columns");
  names.push_back(name);
  types.push_back(t);
  return static_cast<int>(names.size()) - 1;
}

namespace {

DType field_type(const std::vector<Field>& schema, const std::string& name) {
  for (auto& f : schema)
    if (f.name == name) return f.type;
  fail(GFPDB_EINVAL, "column '" + name + "' referenced by the expression is not in the schema");
}

// Type an expression (value expressions only).
DType type_of(const ExprPtr& e, const std::vector<Field>& schema) {
  switch (e->kind) {
    case Expr::Column: return field_type(schema, e->name);
    case Expr::Literal: return e->type;
    case Expr::StrLiteral: return DType::Utf8;
    case Expr::Cast: return e->type;
    case Expr::Arith: {
      DType a = type_of(e->kids[0], schema), b = type_of(e->kids[1], schema);
      if (a == DType::Utf8 || b == DType::Utf8) fail(GFPDB_EINVAL, "arithmetic on utf8");
      if (a == DType::Float64 || b == DType::Float64) return DType::Float64;
      if (a == DType::Int64 || b == DType::Int64) return DType::Int64;
      return DType::Int32;  // int32 / date32 arithmetic stays 32-bit
    }
    case Expr::DateExtract: {
      const DType a = type_of(e->kids[0], schema);
      if (a != DType::Date32 && a != DType::Int32 && a != DType::Int64)
        fail(GFPDB_EINVAL, "DateExtract needs a date: " + expr_to_string(e));
      return DType::Int64;  // extractDay / Month / Year return int64 (DateExtract.cpp:16-24)
    }
    case Expr::DateAdd: {
      const DType a = type_of(e->kids[0], schema), b = type_of(e->kids[1], schema);
      if ((a != DType::Date32 && a != DType::Int32 && a != DType::Int64) || !is_int_type(b))
        fail(GFPDB_EINVAL, "DateAdd needs a date and an integer: " + expr_to_string(e));
      return DType::Date32;
    }
    case Expr::If: {
      const DType t = type_of(e->kids[1], schema), f = type_of(e->kids[2], schema);
      if (t == DType::Utf8 || f == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "If with utf8 branches");
      if (t == DType::Float64 || f == DType::Float64) return DType::Float64;
      if (t == f) return t;
      return DType::Int64;
    }
    case Expr::Substr: return DType::Utf8;
    default: fail(GFPDB_EINVAL, "boolean expression used as a value: " + expr_to_string(e));
  }
}

ValType vt_of(DType t) { return t == DType::Float64 ? VT_F64 : VT_I64; }

void emit(Program& p, Instr in) {
  if (p.n_instrs >= kMaxInstrs) fail(GFPDB_EUNSUPPORTED, "expression too long for one fused kernel");
  p.instrs[p.n_instrs++] = in;
}

void emit_bool(const ExprPtr& e, const std::vector<Field>& schema, Program& p, ColumnSlots& slots);

// Emit postfix code computing e as type `want`.
void emit_value(const ExprPtr& e, DType want, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  DType have = type_of(e, schema);
  switch (e->kind) {
    case Expr::Column: {
      Instr in{};
      in.op = IO_COL;
      in.col = static_cast<int16_t>(slots.slot_for(e->name, have));
      in.vt = vt_of(have);
      emit(p, in);
      break;
    }
    case Expr::Literal: {
      if (e->lit_null) fail(GFPDB_EUNSUPPORTED, "null literals in arithmetic");
      Instr in{};
      in.op = IO_LIT;
      in.vt = vt_of(have);
      in.imm = e->lit;
      emit(p, in);
      break;
    }
    case Expr::Cast: {
      DType src = type_of(e->kids[0], schema);
      emit_value(e->kids[0], src, schema, p, slots);
      if (src == DType::Float64 && is_int_type(have)) {
        Instr in{};
        in.op = IO_F2I;
        in.vt = VT_I64;
        emit(p, in);
      } else if (is_int_type(src) && have == DType::Float64) {
        Instr in{};
        in.op = IO_I2F;
        in.vt = VT_F64;
        emit(p, in);
      }
      if ((have == DType::Int32 || have == DType::Date32) && (src == DType::Int64 || src == DType::Float64)) {
        Instr in{};
        in.op = IO_WRAP32;
        in.vt = VT_I64;
        emit(p, in);
      }
      break;
    }
    case Expr::Arith: {
      emit_value(e->kids[0], have, schema, p, slots);
      emit_value(e->kids[1], have, schema, p, slots);
      Instr in{};
      in.op = e->arith;
      in.vt = vt_of(have);
      emit(p, in);
      if (have == DType::Int32) {
        Instr w{};
        w.op = IO_WRAP32;
        w.vt = VT_I64;
        emit(p, w);
      }
      break;
    }
    case Expr::DateExtract: {
      emit_value(e->kids[0], DType::Int64, schema, p, slots);
      Instr in{};
      in.op = IO_EXTRACT;
      in.vt = VT_I64;
      in.imm.i = e->interval;
      emit(p, in);
      break;
    }
    case Expr::DateAdd: {
      emit_value(e->kids[0], DType::Int64, schema, p, slots);
      emit_value(e->kids[1], DType::Int64, schema, p, slots);
      Instr in{};
      in.op = IO_DATE_ADD;
      in.vt = VT_I64;
      in.imm.i = e->interval;
      emit(p, in);
      break;
    }
    case Expr::If: {
      emit_bool(e->kids[0], schema, p, slots);
      emit_value(e->kids[1], have, schema, p, slots);
      emit_value(e->kids[2], have, schema, p, slots);
      Instr in{};
      in.op = IO_SELECT;
      in.vt = vt_of(have);
      emit(p, in);
      break;
    }
    default: fail(GFPDB_EINVAL, "not a value expression: " + expr_to_string(e));
  }
  // Promote to the requested type.
  if (vt_of(want) == VT_F64 && vt_of(have) == VT_I64) {
    Instr in{};
    in.op = IO_I2F;
    in.vt = VT_F64;
    emit(p, in);
  }
}

Operand operand_for(const ExprPtr& e, DType want, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  DType have = type_of(e, schema);
  Operand o{};
  o.vt = vt_of(want);
  if (e->kind == Expr::Column && vt_of(have) == vt_of(want) && have != DType::Utf8) {
    o.kind = OPND_COL;
    o.col = static_cast<int16_t>(slots.slot_for(e->name, have));
    return o;
  }
  if (e->kind == Expr::Literal) {
    if (e->lit_null) fail(GFPDB_EUNSUPPORTED, "comparison with a null literal");
    o.kind = OPND_LIT;
    if (vt_of(want) == VT_F64 && vt_of(have) == VT_I64) o.lit.f = static_cast<double>(e->lit.i);
    else o.lit = e->lit;
    return o;
  }
  o.kind = OPND_PROG;
  o.prog_begin = static_cast<int16_t>(p.n_instrs);
  emit_value(e, want, schema, p, slots);
  o.prog_len = static_cast<int16_t>(p.n_instrs - o.prog_begin);
  // The device evaluates programs on a fixed stack of kStackDepth values:
  // check the depth here so a kernel can never index past it.
  int depth = 0, max_depth = 0;
  for (int pc = o.prog_begin; pc < o.prog_begin + o.prog_len; ++pc) {
    const int op = p.instrs[pc].op;
    if (op == IO_COL || op == IO_LIT || op == IO_STR_TEST) ++depth;
    else if (op == IO_ADD || op == IO_SUB || op == IO_MUL || op == IO_DIV || op == IO_DATE_ADD || op == IO_CMP ||
             op == IO_AND || op == IO_OR)
      --depth;
    else if (op == IO_SELECT)
      depth -= 2;
    if (depth < 1) fail(GFPDB_EINVAL, "internal: malformed arithmetic program");
    max_depth = std::max(max_depth, depth);
  }
  if (depth != 1) fail(GFPDB_EINVAL, "internal: malformed arithmetic program");
  if (max_depth > kStackDepth) fail(GFPDB_EUNSUPPORTED, "arithmetic expression nests too deeply for one kernel");
  return o;
}

using Clause = std::vector<Leaf>;
using Cnf = std::vector<Clause>;

Leaf const_leaf(bool v) {
  Leaf l{};
  l.op = v ? LO_TRUE : LO_FALSE;
  return l;
}

Cnf cross(const Cnf& a, const Cnf& b) {
  Cnf out;
  for (auto& ca : a)
    for (auto& cb : b) {
      Clause c = ca;
      c.insert(c.end(), cb.begin(), cb.end());
      out.push_back(std::move(c));
      if (out.size() > 256) fail(GFPDB_EUNSUPPORTED, "predicate too complex (CNF blow-up)");
    }
  return out;
}

// String literals live in the program's pool; Program::pad holds the number
// of pool bytes used so far. Returns the literal's first pool byte.
int pool_add(Program& p, const std::string& s) {
  const int used = p.pad;
  if (used + static_cast<int>(s.size()) > kStrPool) fail(GFPDB_EUNSUPPORTED, "string literals exceed the pool");
  std::memcpy(p.strpool + used, s.data(), s.size());
  p.pad = used + static_cast<int>(s.size());
  return used;
}

// The string side of a string test: a utf8 column, or SUBSTRING of one with
// integer literal bounds (Substr.cpp: substr(expr, fromLit, forLit)).
struct StringSide {
  int slot;
  bool sub = false;
  int from = 0, len = 0;
};

StringSide string_side(const ExprPtr& e, const std::vector<Field>& schema, ColumnSlots& slots) {
  StringSide side{};
  ExprPtr col = e;
  if (e->kind == Expr::Substr) {
    const ExprPtr& f = e->kids[1];
    const ExprPtr& n = e->kids[2];
    if (f->kind != Expr::Literal || n->kind != Expr::Literal || f->lit_null || n->lit_null || !is_int_type(f->type) ||
        !is_int_type(n->type))
      fail(GFPDB_EUNSUPPORTED, "Substr takes integer literal bounds: " + expr_to_string(e));
    if (n->lit.i < 0) fail(GFPDB_EINVAL, "Substr length is negative: " + expr_to_string(e));
    if (f->lit.i < -32768 || f->lit.i > 32767 || n->lit.i > 65535)
      fail(GFPDB_EUNSUPPORTED, "Substr bounds out of range: " + expr_to_string(e));
    side.sub = true;
    side.from = static_cast<int>(f->lit.i);
    side.len = static_cast<int>(n->lit.i);
    col = e->kids[0];
  }
  if (col->kind != Expr::Column || field_type(schema, col->name) != DType::Utf8)
    fail(GFPDB_EUNSUPPORTED, "string comparison needs a utf8 column operand: " + expr_to_string(e));
  side.slot = slots.slot_for(col->name, DType::Utf8);
  return side;
}

Leaf string_test_leaf(const ExprPtr& colexpr, const std::string& s, LeafOp op, const std::vector<Field>& schema,
                      Program& p, ColumnSlots& slots) {
  const StringSide side = string_side(colexpr, schema, slots);
  Leaf l{};
  l.op = op;
  l.lhs.kind = OPND_COL;
  l.lhs.col = static_cast<int16_t>(side.slot);
  if (side.sub) {
    l.rhs.col = 1;
    l.rhs.prog_begin = static_cast<int16_t>(side.from);
    l.rhs.prog_len = static_cast<int16_t>(side.len > 32767 ? 32767 : side.len);
  }
  l.str_begin = static_cast<int16_t>(pool_add(p, s));
  l.str_len = static_cast<int16_t>(s.size());
  return l;
}

Leaf string_leaf(const ExprPtr& colexpr, const std::string& s, bool eq, const std::vector<Field>& schema, Program& p,
                 ColumnSlots& slots) {
  return string_test_leaf(colexpr, s, eq ? LO_STR_EQ : LO_STR_NE, schema, p, slots);
}

// Like(left, right) (Like.cpp): a utf8 column or substring against a
// pattern literal.
Leaf like_leaf(const ExprPtr& e, bool neg, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  const ExprPtr& pat = e->kids[1];
  if (pat->kind != Expr::StrLiteral || pat->lit_null) fail(GFPDB_EUNSUPPORTED, "Like needs a pattern literal");
  return string_test_leaf(e->kids[0], pat->str, neg ? LO_NOT_LIKE : LO_LIKE, schema, p, slots);
}

void emit_string_test(const Leaf& l, Program& p) {
  Instr in{};
  in.op = IO_STR_TEST;
  in.vt = VT_I64;
  in.col = l.lhs.col;
  in.imm.i = static_cast<int64_t>(static_cast<uint8_t>(l.op)) | (static_cast<int64_t>(l.str_begin) << 8) |
             (static_cast<int64_t>(l.str_len) << 24) | (l.rhs.col == 1 ? (int64_t{1} << 40) : 0);
  in.pad = static_cast<int32_t>((static_cast<uint32_t>(static_cast<uint16_t>(l.rhs.prog_begin)) << 16) |
                                static_cast<uint16_t>(l.rhs.prog_len));
  emit(p, in);
}

// Push 0 / 1 for a boolean expression (the condition of an If).
void emit_bool(const ExprPtr& e, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  auto lit = [&](int64_t v) {
    Instr in{};
    in.op = IO_LIT;
    in.vt = VT_I64;
    in.imm.i = v;
    emit(p, in);
  };
  auto op0 = [&](InstrOp o) {
    Instr in{};
    in.op = o;
    in.vt = VT_I64;
    emit(p, in);
  };
  switch (e->kind) {
    case Expr::And:
    case Expr::Or:
      for (size_t i = 0; i < e->kids.size(); ++i) {
        emit_bool(e->kids[i], schema, p, slots);
        if (i > 0) op0(e->kind == Expr::And ? IO_AND : IO_OR);
      }
      return;
    case Expr::Not:
      emit_bool(e->kids[0], schema, p, slots);
      op0(IO_NOT);
      return;
    case Expr::Like:
      emit_string_test(like_leaf(e, false, schema, p, slots), p);
      return;
    case Expr::Literal:
      if (!e->is_bool) fail(GFPDB_EINVAL, "numeric literal used as a condition");
      lit(e->lit.i != 0 ? 1 : 0);
      return;
    case Expr::IsNull: lit(0); return;
    case Expr::In: {
      const size_t n = e->type == DType::Utf8 ? e->in_strs.size() : e->in_values.size();
      if (n == 0) {
        lit(0);
        return;
      }
      for (size_t i = 0; i < n; ++i) {
        auto cmp = std::make_shared<Expr>();
        cmp->kind = Expr::Compare;
        cmp->cmp = LO_EQ;
        auto v = std::make_shared<Expr>();
        if (e->type == DType::Utf8) {
          v->kind = Expr::StrLiteral;
          v->str = e->in_strs[i];
        } else {
          v->kind = Expr::Literal;
          v->type = e->type;
          v->lit = e->in_values[i];
        }
        cmp->kids = {e->kids[0], v};
        emit_bool(cmp, schema, p, slots);
        if (i > 0) op0(IO_OR);
      }
      return;
    }
    case Expr::Compare: {
      const ExprPtr& a = e->kids[0];
      const ExprPtr& b = e->kids[1];
      const DType ta = type_of(a, schema), tb = type_of(b, schema);
      if (ta == DType::Utf8 || tb == DType::Utf8) {
        if (e->cmp != LO_EQ && e->cmp != LO_NE) fail(GFPDB_EUNSUPPORTED, "only = and != compare strings");
        const bool eq = e->cmp == LO_EQ;
        if (b->kind == Expr::StrLiteral) emit_string_test(string_leaf(a, b->str, eq, schema, p, slots), p);
        else if (a->kind == Expr::StrLiteral) emit_string_test(string_leaf(b, a->str, eq, schema, p, slots), p);
        else fail(GFPDB_EUNSUPPORTED, "a string comparison in a condition needs a string literal operand");
        return;
      }
      const DType ct = (ta == DType::Float64 || tb == DType::Float64) ? DType::Float64 : DType::Int64;
      emit_value(a, ct, schema, p, slots);
      emit_value(b, ct, schema, p, slots);
      Instr in{};
      in.op = IO_CMP;
      in.vt = vt_of(ct);
      in.imm.i = e->cmp;
      emit(p, in);
      return;
    }
    default: fail(GFPDB_EINVAL, "not a boolean expression: " + expr_to_string(e));
  }
}

Leaf compare_leaf(const ExprPtr& e, LeafOp op, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  const ExprPtr& a = e->kids[0];
  const ExprPtr& b = e->kids[1];
  DType ta = type_of(a, schema), tb = type_of(b, schema);
  if (ta == DType::Utf8 || tb == DType::Utf8) {
    if (op != LO_EQ && op != LO_NE) fail(GFPDB_EUNSUPPORTED, "only = and != compare strings");
    if (a->kind == Expr::StrLiteral) return string_leaf(b, a->str, op == LO_EQ, schema, p, slots);
    if (b->kind == Expr::StrLiteral) return string_leaf(a, b->str, op == LO_EQ, schema, p, slots);
    if (a->kind == Expr::Substr || b->kind == Expr::Substr)
      fail(GFPDB_EUNSUPPORTED, "a substring compares with a string literal");
    if (a->kind == Expr::Column && b->kind == Expr::Column && ta == DType::Utf8 && tb == DType::Utf8) {
      Leaf l{};
      l.op = op == LO_EQ ? LO_STRCOL_EQ : LO_STRCOL_NE;
      l.lhs.kind = OPND_COL;
      l.lhs.col = static_cast<int16_t>(slots.slot_for(a->name, DType::Utf8));
      l.rhs.kind = OPND_COL;
      l.rhs.col = static_cast<int16_t>(slots.slot_for(b->name, DType::Utf8));
      return l;
    }
    fail(GFPDB_EUNSUPPORTED, "string comparison needs a string literal or two string columns");
  }
  DType ct = (ta == DType::Float64 || tb == DType::Float64) ? DType::Float64 : DType::Int64;
  Leaf l{};
  l.op = op;
  l.cmp_vt = vt_of(ct);
  l.lhs = operand_for(a, ct, schema, p, slots);
  l.rhs = operand_for(b, ct, schema, p, slots);
  return l;
}

Cnf to_cnf(const ExprPtr& e, bool neg, const std::vector<Field>& schema, Program& p, ColumnSlots& slots) {
  switch (e->kind) {
    case Expr::And:
    case Expr::Or: {
      bool conj = (e->kind == Expr::And) != neg;
      Cnf acc;
      bool first = true;
      for (auto& k : e->kids) {
        Cnf c = to_cnf(k, neg, schema, p, slots);
        if (conj) {
          acc.insert(acc.end(), c.begin(), c.end());
        } else {
          acc = first ? c : cross(acc, c);
        }
        first = false;
      }
      return acc;
    }
    case Expr::Not: return to_cnf(e->kids[0], !neg, schema, p, slots);
    case Expr::Compare: {
      LeafOp op = neg ? negate(e->cmp) : e->cmp;
      return Cnf{Clause{compare_leaf(e, op, schema, p, slots)}};
    }
    case Expr::In: {
      const ExprPtr& x = e->kids[0];
      Clause eqs;
      Cnf nes;
      size_t n = e->type == DType::Utf8 ? e->in_strs.size() : e->in_values.size();
      if (n == 0) return Cnf{Clause{const_leaf(neg)}};
      for (size_t i = 0; i < n; ++i) {
        auto cmp = std::make_shared<Expr>();
        cmp->kind = Expr::Compare;
        cmp->cmp = LO_EQ;
        auto litn = std::make_shared<Expr>();
        if (e->type == DType::Utf8) {
          litn->kind = Expr::StrLiteral;
          litn->str = e->in_strs[i];
        } else {
          litn->kind = Expr::Literal;
          litn->type = e->type;
          litn->lit = e->in_values[i];
        }
        cmp->kids = {x, litn};
        Leaf l = compare_leaf(cmp, neg ? LO_NE : LO_EQ, schema, p, slots);
        if (neg) nes.push_back(Clause{l});
        else eqs.push_back(l);
      }
      return neg ? nes : Cnf{eqs};
    }
    case Expr::IsNull:
      // Inputs carry no nulls (nullable inputs are rejected at import), so
      // IsNull is false for every row.
      return Cnf{Clause{const_leaf(neg)}};
    case Expr::Like: return Cnf{Clause{like_leaf(e, neg, schema, p, slots)}};
    case Expr::Literal:
      if (!e->is_bool) fail(GFPDB_EINVAL, "numeric literal used as a predicate");
      return Cnf{Clause{const_leaf((e->lit.i != 0) != neg)}};
    default: fail(GFPDB_EINVAL, "not a boolean expression: " + expr_to_string(e));
  }
}

}  // namespace

CompiledPredicate compile_predicate(const ExprPtr& e, const std::vector<Field>& schema) {
  CompiledPredicate cp;
  std::memset(&cp.prog, 0, sizeof(cp.prog));
  cp.text = expr_to_string(e);
  Cnf cnf = to_cnf(e, false, schema, cp.prog, cp.slots);
  // Simplify: drop clauses holding a TRUE leaf, drop FALSE leaves.
  Cnf simp;
  bool always_false = false;
  for (auto& c : cnf) {
    bool taut = false;
    Clause kept;
    for (auto& l : c) {
      if (l.op == LO_TRUE) taut = true;
      else if (l.op != LO_FALSE) kept.push_back(l);
    }
    if (taut) continue;
    if (kept.empty()) always_false = true;
    simp.push_back(std::move(kept));
  }
  if (always_false) simp = Cnf{Clause{const_leaf(false)}};
  if (static_cast<int>(simp.size()) > kMaxClauses) fail(GFPDB_EUNSUPPORTED, "predicate has too many clauses");
  int nl = 0;
  cp.prog.n_clauses = static_cast<int32_t>(simp.size());
  for (size_t c = 0; c < simp.size(); ++c) {
    cp.prog.clause_begin[c] = static_cast<int16_t>(nl);
    for (auto& l : simp[c]) {
      if (nl >= kMaxLeaves) fail(GFPDB_EUNSUPPORTED, "predicate has too many comparisons");
      cp.prog.leaves[nl++] = l;
    }
  }
  cp.prog.clause_begin[simp.size()] = static_cast<int16_t>(nl);
  cp.prog.n_leaves = nl;
  return cp;
}

bool utf8_source(const ExprPtr& e, const std::vector<Field>& schema, Utf8Source* out) {
  if (type_of(e, schema) != DType::Utf8) return false;
  ColumnSlots scratch;
  const StringSide side = string_side(e, schema, scratch);
  out->column = scratch.names.at(side.slot);
  out->sub = side.sub;
  out->from = side.from;
  out->len = side.len;
  return true;
}

Operand compile_value(const ExprPtr& e, const std::vector<Field>& schema, Program& prog, ColumnSlots& slots,
                      DType* result_type) {
  DType t = type_of(e, schema);
  if (t == DType::Utf8) fail(GFPDB_EUNSUPPORTED, "utf8 aggregate input");
  // Aggregates over int32/int64/date32 inputs are summed in int64.
  DType want = t == DType::Float64 ? DType::Float64 : DType::Int64;
  if (result_type) *result_type = t;
  return operand_for(e, want, schema, prog, slots);
}

void bind_columns(const ColumnSlots& slots, const TupleSet& ts, DevCol* out, int max_cols) {
  if (static_cast<int>(slots.names.size()) > max_cols) fail(GFPDB_EUNSUPPORTED, "too many columns");
  for (size_t i = 0; i < slots.names.size(); ++i) {
    int ci = ts.require_column(slots.names[i]);
    const auto& c = ts.column(ci);
    if (c->type != slots.types[i])
      fail(GFPDB_EINVAL, "column '" + slots.names[i] + "' changed type since the expression was compiled");
    out[i].data = c->data;
    out[i].offsets = c->offsets;
    out[i].type = static_cast<int32_t>(c->type);
    out[i].pad = 0;
  }
}

}  // namespace gfpdb
