// Expression trees and their lowering to device programs.
//
// The node kinds and JSON field names follow the reference's expression
// language (fpdb-expression-gandiva/include/fpdb/expression/gandiva/ExpressionType.h:10-35;
// Expression::fromJson, fpdb-expression-gandiva/src/Expression.cpp:52-148):
// "Column"{columnName}, "NumericLiteral"{dataType,value}, "StringLiteral"{value},
// "And"/"Or"{exprs}, "Not"/"IsNull"{expr}, "Cast"{expr,dataType},
// "In"{expr,values,dataType}, and the binary nodes {left,right}: EqualTo,
// NotEqualTo, LessThan, LessThanOrEqualTo, GreaterThan, GreaterThanOrEqualTo,
// Add, Subtract, Multiply, Divide. dataType is a type name ("int32", "int64",
// "float64", "date32", "boolean", "utf8") instead of the reference's
// serialised arrow::DataType bytes.
//
// Typing follows BinaryExpression::castGandivaExprToUpperType
// (fpdb-expression-gandiva/src/BinaryExpression.cpp:57-102): int32 op int64
// is computed in int64, int op double in double, and same-type arithmetic
// stays in that type (int32 * int32 wraps to int32 as Gandiva's multiply does).
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "../program.h"
#include "json.h"
#include "tupleset.h"

namespace gfpdb {

struct Expr;
using ExprPtr = std::shared_ptr<const Expr>;

struct Expr {
  enum Kind { Column, Literal, StrLiteral, And, Or, Not, Compare, Arith, Cast, In, IsNull,
              DateExtract, DateAdd, If, Like, Substr };
  Kind kind = Literal;
  std::string name;                 // Column
  DType type = DType::Int64;        // Literal type / Cast target / In element type
  bool is_bool = false;             // boolean literal
  Scalar lit{};                     // numeric literal (is_bool: lit.i = 0/1)
  bool lit_null = false;            // literal without a value
  std::string str;                  // StrLiteral
  LeafOp cmp = LO_EQ;               // Compare
  InstrOp arith = IO_ADD;           // Arith
  std::vector<ExprPtr> kids;
  int interval = 0;                 // DateExtract / DateAdd: 0 Day, 1 Month, 2 Year
  std::vector<Scalar> in_values;    // In over numbers
  std::vector<std::string> in_strs; // In over strings
};

ExprPtr parse_expr(const json::Value& v);
ExprPtr parse_expr_json(const std::string& text);
std::string expr_to_string(const ExprPtr& e);
void expr_columns(const ExprPtr& e, std::vector<std::string>& out);  // distinct, first-use order

// Column slots referenced by a program: slot i is column `names[i]`.
struct ColumnSlots {
  std::vector<std::string> names;
  std::vector<DType> types;
  int slot_for(const std::string& name, DType t);
};

struct CompiledPredicate {
  Program prog{};
  ColumnSlots slots;
  std::string text;
};

// Lower a boolean expression to CNF over the given schema.
CompiledPredicate compile_predicate(const ExprPtr& e, const std::vector<Field>& schema);

// Lower a value expression to an operand (columns, literals, or a postfix
// program appended to prog.instrs). Returns the operand and its result type.
// A utf8-valued expression a projection produces: a utf8 column, or
// SUBSTRING of one with integer literal bounds (Substr.cpp). Returns false
// when `e` is not utf8-valued; fails when it is but has another form.
struct Utf8Source {
  std::string column;
  bool sub = false;
  int from = 0, len = 0;
};
bool utf8_source(const ExprPtr& e, const std::vector<Field>& schema, Utf8Source* out);

Operand compile_value(const ExprPtr& e, const std::vector<Field>& schema, Program& prog, ColumnSlots& slots,
                      DType* result_type);

// Resolve program column slots against a TupleSet.
void bind_columns(const ColumnSlots& slots, const TupleSet& ts, DevCol* out, int max_cols);

}  // namespace gfpdb
