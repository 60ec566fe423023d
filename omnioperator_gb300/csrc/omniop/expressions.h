// Expression trees for join filters.
//
// The node classes mirror the reference's (expression/expressions.h:22-62 and the FieldExpr,
// LiteralExpr, BinaryExpr, UnaryExpr and IsNullExpr classes): a FieldExpr names a column of the
// joined row (probe columns first, then build columns, as LookupJoinOperator numbers them,
// lookup_join.cpp:215-240), a BinaryExpr owns its two children.  The GB300 join compiles a
// filter tree into a postfix program that the probe kernel runs per candidate pair
// (CompileJoinFilter in host/hash_join.cpp); comparisons, NOT, AND, OR, IS [NOT] NULL and
// arithmetic over fixed-width integer-like and double columns and literals, VARCHAR/CHAR columns
// and literals, the substr function (a FuncExpr), IF, CASE (SwitchExpr), IN, BETWEEN and
// COALESCE are supported, anything else is refused
// with EXPRESSION_NOT_SUPPORT as the reference refuses expressions its code generator cannot
// handle (lookup_join.cpp:175-187).
#pragma once

#include <cstdint>
#include <string>
#include <utility>
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

// Conditional and set nodes (expressions.h:166-230), owning their children; their return
// types follow the reference's constructors (expressions.cpp:211-276).
class InExpr : public Expr {
public:
    explicit InExpr(std::vector<Expr *> args) : Expr(type::BooleanType()), arguments(std::move(args)) {}
    ~InExpr() override { DeleteExprs(arguments); }
    InExpr(const InExpr &) = delete;
    InExpr &operator=(const InExpr &) = delete;
    ExprType GetType() const override { return ExprType::IN_E; }
    std::vector<Expr *> arguments;  // the value, then the list
};

class BetweenExpr : public Expr {
public:
    BetweenExpr(Expr *val, Expr *lowBound, Expr *upBound)
        : Expr(type::BooleanType()), value(val), lowerBound(lowBound), upperBound(upBound)
    {}
    ~BetweenExpr() override
    {
        delete value;
        delete lowerBound;
        delete upperBound;
    }
    BetweenExpr(const BetweenExpr &) = delete;
    BetweenExpr &operator=(const BetweenExpr &) = delete;
    ExprType GetType() const override { return ExprType::BETWEEN_E; }
    Expr *value;
    Expr *lowerBound;
    Expr *upperBound;
};

class IfExpr : public Expr {
public:
    IfExpr(Expr *cond, Expr *texp, Expr *fexp)
        : Expr(texp->GetReturnType()), condition(cond), trueExpr(texp), falseExpr(fexp)
    {}
    ~IfExpr() override
    {
        delete condition;
        delete trueExpr;
        delete falseExpr;
    }
    IfExpr(const IfExpr &) = delete;
    IfExpr &operator=(const IfExpr &) = delete;
    ExprType GetType() const override { return ExprType::IF_E; }
    Expr *condition;
    Expr *trueExpr;
    Expr *falseExpr;
};

class SwitchExpr : public Expr {
public:
    SwitchExpr(std::vector<std::pair<Expr *, Expr *>> whens, Expr *fexp)
        : Expr(fexp->GetReturnType()), whenClause(std::move(whens)), falseExpr(fexp)
    {}
    ~SwitchExpr() override
    {
        for (auto &w : whenClause) {
            delete w.first;
            delete w.second;
        }
        delete falseExpr;
    }
    SwitchExpr(const SwitchExpr &) = delete;
    SwitchExpr &operator=(const SwitchExpr &) = delete;
    ExprType GetType() const override { return ExprType::SWITCH_E; }
    std::vector<std::pair<Expr *, Expr *>> whenClause;
    Expr *falseExpr;
};

class CoalesceExpr : public Expr {
public:
    CoalesceExpr(Expr *val1, Expr *val2) : Expr(val1->GetReturnType()), value1(val1), value2(val2) {}
    ~CoalesceExpr() override
    {
        delete value1;
        delete value2;
    }
    CoalesceExpr(const CoalesceExpr &) = delete;
    CoalesceExpr &operator=(const CoalesceExpr &) = delete;
    ExprType GetType() const override { return ExprType::COALESCE_E; }
    Expr *value1;
    Expr *value2;
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
