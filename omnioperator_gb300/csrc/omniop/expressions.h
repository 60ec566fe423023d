// Expression trees for join filters.
//
// The node classes mirror the reference's (expression/expressions.h:22-62 and the FieldExpr,
// LiteralExpr, BinaryExpr, UnaryExpr and IsNullExpr classes): a FieldExpr names a column of the
// joined row (probe columns first, then build columns, as LookupJoinOperator numbers them,
// lookup_join.cpp:215-240), a BinaryExpr owns its two children.  The GB300 join compiles a
// filter tree into a postfix program that the probe kernel runs per candidate pair
// (CompileJoinFilter in host/hash_join.cpp); comparisons, NOT, AND, OR, IS [NOT] NULL and
// arithmetic over fixed-width integer-like and double columns and literals, VARCHAR/CHAR columns
// and literals, and the substr function (a FuncExpr) are supported, anything else is refused
// with EXPRESSION_NOT_SUPPORT as the reference refuses expressions its code generator cannot
// handle (lookup_join.cpp:175-187).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "types.h"

namespace omniruntime {
namespace expressions {

enum class Operator {
    EQ, NEQ, LT, LTE, GT, GTE,
    AND, OR, NOT,
    ADD, SUB, MUL, DIV, MOD, TRY_ADD, TRY_SUB, TRY_MUL, TRY_DIV,
    INVALIDOP
};

enum class ExprType {
    LITERAL_E, FIELD_E, BINARY_E, UNARY_E, IN_E, BETWEEN_E, IF_E, SWITCH_E, COALESCE_E, IS_NULL_E, FUNC_E, INVALID_E
};

class Expr {
public:
    explicit Expr(type::DataTypePtr t) : dataType(std::move(t)) {}
    virtual ~Expr() = default;
    virtual ExprType GetType() const = 0;
    type::DataTypePtr GetReturnType() const { return dataType; }
    static void DeleteExprs(const std::vector<Expr *> &exprs)
    {
        for (auto *e : exprs) {
            delete e;
        }
    }

    type::DataTypePtr dataType;
};

class FieldExpr : public Expr {
public:
    FieldExpr(int32_t colVal, type::DataTypePtr t) : Expr(std::move(t)), colVal(colVal) {}
    ExprType GetType() const override { return ExprType::FIELD_E; }
    int32_t colVal;
};

class LiteralExpr : public Expr {
public:
    // Integer-like and BOOLEAN literals (the value as int64); isNull for a NULL literal.
    LiteralExpr(int64_t v, type::DataTypePtr t) : Expr(std::move(t)), longVal(v) {}
    LiteralExpr(double v, type::DataTypePtr t) : Expr(std::move(t)), doubleVal(v) {}
    // VARCHAR/CHAR literal; takes ownership of `v`, as the reference's LiteralExpr(std::string *,
    // DataTypePtr) does.
    LiteralExpr(std::string *v, type::DataTypePtr t) : Expr(std::move(t)), stringVal(v) {}
    ~LiteralExpr() override { delete stringVal; }
    LiteralExpr(const LiteralExpr &) = delete;
    LiteralExpr &operator=(const LiteralExpr &) = delete;
    ExprType GetType() const override { return ExprType::LITERAL_E; }
    int64_t longVal = 0;
    double doubleVal = 0.0;
    std::string *stringVal = nullptr;
    bool isNull = false;
};

class BinaryExpr : public Expr {
public:
    BinaryExpr(Operator op, Expr *left, Expr *right, type::DataTypePtr t)
        : Expr(std::move(t)), op(op), left(left), right(right)
    {}
    ~BinaryExpr() override
    {
        delete left;
        delete right;
    }
    ExprType GetType() const override { return ExprType::BINARY_E; }
    Operator op;
    Expr *left;
    Expr *right;
};

class UnaryExpr : public Expr {
public:
    UnaryExpr(Operator op, Expr *exp, type::DataTypePtr t) : Expr(std::move(t)), op(op), exp(exp) {}
    ~UnaryExpr() override { delete exp; }
    ExprType GetType() const override { return ExprType::UNARY_E; }
    Operator op;
    Expr *exp;
};

// A function call by name (expressions.h FuncExpr): owns its arguments.
class FuncExpr : public Expr {
public:
    FuncExpr(std::string fnName, std::vector<Expr *> args, type::DataTypePtr returnType)
        : Expr(std::move(returnType)), funcName(std::move(fnName)), arguments(std::move(args))
    {}
    ~FuncExpr() override { DeleteExprs(arguments); }
    FuncExpr(const FuncExpr &) = delete;
    FuncExpr &operator=(const FuncExpr &) = delete;
    ExprType GetType() const override { return ExprType::FUNC_E; }
    std::string funcName;
    std::vector<Expr *> arguments;
};

class IsNullExpr : public Expr {
public:
    explicit IsNullExpr(Expr *value) : Expr(type::BooleanType()), value(value) {}
    ~IsNullExpr() override { delete value; }
    ExprType GetType() const override { return ExprType::IS_NULL_E; }
    Expr *value;
};

}  // namespace expressions
}  // namespace omniruntime
