// extern "C" boundary (include/omniop_gb300.h).  No exception crosses it: every entry point
// returns a status code and leaves a thread-local message for omg_last_error().
#include "omniop_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "host/gpu_runtime.h"
#include "host/sizer.h"
#include "kernels/agg_noalloc.h"
#include "kernels/launch.h"
#include "omniop/batched_agg.h"
#include "omniop/hash_aggregation.h"
#include "omniop/expressions.h"
#include "omniop/hash_join.h"
#include "omniop/memory.h"
#include "omniop/operator.h"
#include "omniop/vector.h"

using omniruntime::exception::OmniException;
using omniruntime::op::HashAggregationOperator;
using omniruntime::op::HashAggregationOperatorFactory;
using omniruntime::op::HashBuilderOperatorFactory;
using omniruntime::op::LookupJoinOperatorFactory;
using omniruntime::op::Operator;
using omniruntime::op::OperatorFactory;
using omniruntime::type::DataType;
using omniruntime::type::DataTypeId;
using omniruntime::type::DataTypePtr;
using omniruntime::type::DataTypes;
using omniruntime::vec::BaseVector;
using omniruntime::vec::VectorBatch;
using omniruntime::vec::VectorHelper;

namespace {
// Per-thread message of the last failing call, in a fixed buffer so that reporting an error
// never allocates.
thread_local char g_error[512];

void ClearError() { g_error[0] = '\0'; }
void SetError(const char *m) { std::snprintf(g_error, sizeof(g_error), "%s", m); }
void SetError(const std::string &m) { SetError(m.c_str()); }

template <typename F> int32_t Guard(F &&f)
{
    try {
        ClearError();
        f();
        return OMG_OK;
    } catch (const OmniException &e) {
        SetError(e.what());
        return e.GetStatus();
    } catch (const std::bad_alloc &e) {
        SetError(std::string("out of host memory: ") + e.what());
        return OMG_ERR_OOM;
    } catch (const std::exception &e) {
        SetError(e.what());
        return OMG_ERR_INTERNAL;
    } catch (...) {
        SetError("unknown error");
        return OMG_ERR_INTERNAL;
    }
}

void Require(bool cond, const char *msg)
{
    if (!cond) {
        throw OmniException("INVALID_ARGUMENT", msg, OMG_ERR_INVALID_ARG);
    }
}

DataTypePtr ToType(const OmgDataType &t)
{
    return std::make_shared<DataType>(static_cast<DataTypeId>(t.id), t.precision, t.scale, t.width);
}

DataTypes ToTypes(const OmgDataType *t, int32_t n)
{
    std::vector<DataTypePtr> v;
    for (int32_t i = 0; i < n; ++i) {
        v.push_back(ToType(t[i]));
    }
    return DataTypes(v);
}

Operator *AsOp(void *op)
{
    Require(op != nullptr, "null operator handle");
    return static_cast<Operator *>(op);
}
}  // namespace

extern "C" {

const char *omg_last_error(void) { return g_error; }

const char *omg_version(void) { return "omniop-gb300 0.1 (sm_103a)"; }

int32_t omg_device_available(void) { return omg::DeviceAvailable() ? 1 : 0; }

int32_t omg_config_set_policy(int32_t policy)
{
    return Guard([&] {
        Require(policy == OMG_POLICY_SPARK || policy == OMG_POLICY_GENERIC, "unknown policy");
        omniruntime::op::SetSupportContainerVecRule(policy == OMG_POLICY_SPARK
                ? omniruntime::op::SupportContainerVecRule::NOT_SUPPORT
                : omniruntime::op::SupportContainerVecRule::SUPPORT);
    });
}

int32_t omg_config_get_policy(void)
{
    return omniruntime::op::GetSupportContainerVecRule() == omniruntime::op::SupportContainerVecRule::NOT_SUPPORT
        ? OMG_POLICY_SPARK
        : OMG_POLICY_GENERIC;
}

int32_t omg_config_set_substr_rules(int32_t negative_rule, int32_t zero_rule)
{
    return Guard([&] {
        Require((negative_rule == 0 || negative_rule == 1) && (zero_rule == 0 || zero_rule == 1), "unknown rule");
        omniruntime::op::SetNegativeStartIndexOutOfBoundsRule(negative_rule == 1
                ? omniruntime::op::NegativeStartIndexOutOfBoundsRule::INTERCEPT_FROM_BEYOND
                : omniruntime::op::NegativeStartIndexOutOfBoundsRule::EMPTY_STRING);
        omniruntime::op::SetZeroStartIndexSupportRule(zero_rule == 1
                ? omniruntime::op::ZeroStartIndexSupportRule::IS_SUPPORT
                : omniruntime::op::ZeroStartIndexSupportRule::IS_NOT_SUPPORT);
    });
}

int32_t omg_config_get_substr_rules(int32_t *negative_rule, int32_t *zero_rule)
{
    return Guard([&] {
        Require(negative_rule != nullptr && zero_rule != nullptr, "invalid arguments");
        *negative_rule = omniruntime::op::GetNegativeStartIndexOutOfBoundsRule() ==
                omniruntime::op::NegativeStartIndexOutOfBoundsRule::INTERCEPT_FROM_BEYOND
            ? 1
            : 0;
        *zero_rule =
            omniruntime::op::GetZeroStartIndexSupportRule() == omniruntime::op::ZeroStartIndexSupportRule::IS_SUPPORT
            ? 1
            : 0;
    });
}

int32_t omg_debug_fail_next_allocs(int32_t n)
{
    omg::SetFailNextDeviceAllocs(n < 0 ? 0 : n);
    return OMG_OK;
}

int32_t omg_debug_set_wait_budget(int64_t ticks)
{
    omg::SetWaitBudget(ticks < 0 ? 0 : ticks);
    return OMG_OK;
}

int32_t omg_debug_set_staged_probe(int32_t on)
{
    omg::SetStagedProbe(on != 0);
    return OMG_OK;
}

int32_t omg_debug_last_probe_kernel(void) { return omg::LastProbeKernel(); }

int32_t omg_debug_set_fused_training(int32_t on)
{
    omg::SetFusedTraining(on != 0);
    return OMG_OK;
}

int32_t omg_debug_set_bulk_probe(int32_t mode)
{
    return Guard([&] {
        Require(mode >= 0 && mode <= 2, "bulk probe mode must be 0, 1 or 2");
        omg::SetBulkProbe(mode);
    });
}

int32_t omg_debug_set_agg_flush_rows(int64_t rows)
{
    omg::SetAggFlushRows(rows < 0 ? 0 : rows);
    return OMG_OK;
}

int32_t omg_debug_set_probe_chunk_rows(int64_t rows)
{
    omg::SetProbeChunkRows(rows < 0 ? 0 : rows);
    return OMG_OK;
}

// ---- vectors
int32_t omg_vec_new(int32_t type_id, int32_t size, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && size >= 0, "invalid arguments");
        const int32_t w = omniruntime::type::TypeWidth(static_cast<DataTypeId>(type_id));
        Require(w > 0, "unsupported vector type");
        *out_vec = new BaseVector(static_cast<DataTypeId>(type_id), w, size, false);
    });
}

int32_t omg_vec_new_fixed(int32_t width, int32_t size, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && size >= 0 && width > 0, "invalid arguments");
        *out_vec = new BaseVector(omniruntime::type::OMNI_FIXEDBINARY, width, size, false);
    });
}

int32_t omg_vec_new_varchar(int32_t type_id, int32_t size, int64_t data_bytes, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && size >= 0 && data_bytes >= 0 && data_bytes < (int64_t(1) << 31),
            "invalid arguments");
        Require(type_id == omniruntime::type::OMNI_VARCHAR || type_id == omniruntime::type::OMNI_CHAR,
            "not a VARCHAR/CHAR type");
        *out_vec = new BaseVector(static_cast<DataTypeId>(type_id), size, data_bytes, false);
    });
}

int32_t omg_vec_new_dictionary(const int32_t *ids, int32_t size, void *dictionary, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && dictionary != nullptr && size >= 0 && (size == 0 || ids != nullptr),
            "invalid arguments");
        *out_vec = VectorHelper::CreateDictionaryVector(ids, size, *static_cast<BaseVector *>(dictionary));
    });
}

int32_t omg_vec_encoding(void *vec) { return vec ? static_cast<int32_t>(static_cast<BaseVector *>(vec)->GetEncoding()) : -1; }

int32_t omg_vec_num_fields(void *vec) { return vec ? static_cast<BaseVector *>(vec)->NumFields() : -1; }

void *omg_vec_field(void *vec, int32_t i)
{
    auto *v = static_cast<BaseVector *>(vec);
    return v != nullptr && i >= 0 && i < v->NumFields() ? v->Field(i) : nullptr;
}

int32_t *omg_vec_offsets(void *vec) { return vec ? static_cast<BaseVector *>(vec)->RawOffsets() : nullptr; }
int64_t omg_vec_data_bytes(void *vec) { return vec ? static_cast<BaseVector *>(vec)->DataBytes() : -1; }

int32_t omg_vec_new_device(int32_t type_id, int32_t width, int32_t size, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && size >= 0, "invalid arguments");
        omg::RequireDevice();
        const int32_t w = omniruntime::type::TypeWidth(static_cast<DataTypeId>(type_id), width);
        Require(w > 0, "unsupported vector type");
        *out_vec = new BaseVector(static_cast<DataTypeId>(type_id), w, size, true, nullptr);
        omg::CudaCheck(cudaStreamSynchronize(nullptr), "zero device vector");
    });
}

int32_t omg_vec_wrap_device(int32_t type_id, int32_t width, int32_t size, void *values, void *nulls, void **out_vec)
{
    return Guard([&] {
        Require(out_vec != nullptr && size >= 0 && values != nullptr, "invalid arguments");
        const int32_t w = omniruntime::type::TypeWidth(static_cast<DataTypeId>(type_id), width);
        Require(w > 0, "unsupported vector type");
        auto vb = omg::Buffer::DeviceView(values, static_cast<size_t>(w) * size);
        omg::BufferPtr nb = nulls != nullptr ? omg::Buffer::DeviceView(nulls, (size + 7) / 8) : nullptr;
        *out_vec = new BaseVector(static_cast<DataTypeId>(type_id), w, size, vb, 0, nb, 0, nulls != nullptr);
    });
}

int32_t omg_vec_free(void *vec)
{
    return Guard([&] { delete static_cast<BaseVector *>(vec); });
}

void *omg_vec_values(void *vec) { return vec ? static_cast<BaseVector *>(vec)->RawValues() : nullptr; }
uint8_t *omg_vec_nulls(void *vec) { return vec ? static_cast<BaseVector *>(vec)->RawNulls() : nullptr; }
int32_t omg_vec_size(void *vec) { return vec ? static_cast<BaseVector *>(vec)->GetSize() : -1; }
int32_t omg_vec_type(void *vec) { return vec ? static_cast<BaseVector *>(vec)->GetTypeId() : -1; }
int32_t omg_vec_width(void *vec) { return vec ? static_cast<BaseVector *>(vec)->GetWidth() : -1; }
int32_t omg_vec_is_device(void *vec) { return vec ? (static_cast<BaseVector *>(vec)->IsDevice() ? 1 : 0) : -1; }
int32_t omg_vec_has_null(void *vec) { return vec ? (static_cast<BaseVector *>(vec)->HasNull() ? 1 : 0) : -1; }
int32_t omg_vec_set_null_flag(void *vec, int32_t has_null)
{
    return Guard([&] {
        Require(vec != nullptr, "null vector");
        static_cast<BaseVector *>(vec)->SetNullFlag(has_null != 0);
    });
}

// ---- batches
int32_t omg_batch_new(int32_t row_count, void **out_batch)
{
    return Guard([&] {
        Require(out_batch != nullptr && row_count >= 0, "invalid arguments");
        *out_batch = new VectorBatch(row_count);
    });
}

int32_t omg_batch_append(void *batch, void *vec)
{
    return Guard([&] {
        Require(batch != nullptr && vec != nullptr, "null handle");
        static_cast<VectorBatch *>(batch)->Append(static_cast<BaseVector *>(vec));
    });
}

void *omg_batch_get(void *batch, int32_t index)
{
    auto *b = static_cast<VectorBatch *>(batch);
    if (b == nullptr || index < 0 || index >= b->GetVectorCount()) {
        return nullptr;
    }
    return b->Get(index);
}

int32_t omg_batch_row_count(void *batch) { return batch ? static_cast<VectorBatch *>(batch)->GetRowCount() : -1; }
int32_t omg_batch_vector_count(void *batch)
{
    return batch ? static_cast<VectorBatch *>(batch)->GetVectorCount() : -1;
}

int32_t omg_batch_free(void *batch)
{
    return Guard([&] { VectorHelper::FreeVecBatch(static_cast<VectorBatch *>(batch)); });
}

int32_t omg_batch_to_device(void *batch, void **out_batch)
{
    return Guard([&] {
        Require(batch != nullptr && out_batch != nullptr, "null handle");
        omg::RequireDevice();
        *out_batch = VectorHelper::CopyBatch(static_cast<VectorBatch *>(batch), true, nullptr);
    });
}

int32_t omg_batch_to_host(void *batch, void **out_batch)
{
    return Guard([&] {
        Require(batch != nullptr && out_batch != nullptr, "null handle");
        omg::RequireDevice();
        *out_batch = VectorHelper::CopyBatch(static_cast<VectorBatch *>(batch), false, nullptr);
    });
}

// ---- factories
int32_t omg_hashagg_factory_create(const uint32_t *group_cols, const OmgDataType *group_types, int32_t n_group,
    const uint32_t *agg_func_types, int32_t n_agg, const int32_t *agg_col_offsets, const uint32_t *agg_cols,
    const OmgDataType *agg_input_types, const int32_t *agg_out_offsets, const OmgDataType *agg_output_types,
    const int32_t *mask_cols, const uint8_t *input_raws, const uint8_t *output_partials, int32_t overflow_as_null,
    void **out_factory)
{
    return Guard([&] {
        Require(out_factory != nullptr && n_group >= 0 && n_agg >= 0, "invalid arguments");
        Require(n_group == 0 || (group_cols != nullptr && group_types != nullptr), "null group arrays");
        Require(n_agg == 0 || (agg_func_types != nullptr && agg_col_offsets != nullptr && agg_out_offsets != nullptr),
            "null aggregator arrays");
        std::vector<uint32_t> groupCols(group_cols, group_cols + n_group);
        DataTypes groupTypes = ToTypes(group_types, n_group);
        std::vector<std::vector<uint32_t>> aggCols;
        std::vector<DataTypes> aggIn;
        std::vector<DataTypes> aggOut;
        std::vector<uint32_t> funcs(agg_func_types, agg_func_types + n_agg);
        std::vector<uint32_t> masks;
        std::vector<bool> raws;
        std::vector<bool> partials;
        for (int32_t i = 0; i < n_agg; ++i) {
            const int32_t a0 = agg_col_offsets[i];
            const int32_t a1 = agg_col_offsets[i + 1];
            Require(a1 >= a0, "bad aggregator column offsets");
            aggCols.emplace_back(agg_cols + a0, agg_cols + a1);
            aggIn.push_back(ToTypes(agg_input_types + a0, a1 - a0));
            const int32_t o0 = agg_out_offsets[i];
            const int32_t o1 = agg_out_offsets[i + 1];
            Require(o1 >= o0, "bad aggregator output offsets");
            aggOut.push_back(ToTypes(agg_output_types + o0, o1 - o0));
            masks.push_back(mask_cols == nullptr || mask_cols[i] < 0 ? UINT32_MAX : static_cast<uint32_t>(mask_cols[i]));
            raws.push_back(input_raws == nullptr ? true : input_raws[i] != 0);
            partials.push_back(output_partials == nullptr ? false : output_partials[i] != 0);
        }
        auto *f = new HashAggregationOperatorFactory(groupCols, groupTypes, aggCols, aggIn, aggOut, funcs, masks, raws,
            partials, overflow_as_null != 0);
        try {
            f->Init();
        } catch (...) {
            delete f;
            throw;
        }
        *out_factory = static_cast<OperatorFactory *>(f);
    });
}

int32_t omg_hashbuilder_factory_create(int32_t join_type, const OmgDataType *build_types, int32_t n_build_types,
    const int32_t *build_hash_cols, int32_t n_hash_cols, int32_t operator_count, void **out_factory)
{
    return Guard([&] {
        Require(out_factory != nullptr && build_types != nullptr && n_build_types > 0, "invalid arguments");
        auto *f = HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(
            static_cast<omniruntime::op::JoinType>(join_type), ToTypes(build_types, n_build_types), build_hash_cols,
            n_hash_cols, operator_count);
        *out_factory = static_cast<OperatorFactory *>(f);
    });
}

int32_t omg_hashbuilder_factory_create_side(int32_t join_type, int32_t build_side, const OmgDataType *build_types,
    int32_t n_build_types, const int32_t *build_hash_cols, int32_t n_hash_cols, int32_t operator_count,
    void **out_factory)
{
    return Guard([&] {
        Require(out_factory != nullptr && build_types != nullptr && n_build_types > 0, "invalid arguments");
        auto *f = HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(
            static_cast<omniruntime::op::JoinType>(join_type), static_cast<omniruntime::op::BuildSide>(build_side),
            ToTypes(build_types, n_build_types), build_hash_cols, n_hash_cols, operator_count);
        *out_factory = static_cast<OperatorFactory *>(f);
    });
}

int32_t omg_lookupouterjoin_factory_create(const OmgDataType *probe_types, int32_t n_probe_types,
    const int32_t *probe_output_cols, int32_t n_probe_output, const int32_t *build_output_cols, int32_t n_build_output,
    const OmgDataType *build_output_types, int64_t hash_builder_factory_addr, int32_t build_side, void **out_factory)
{
    return Guard([&] {
        Require(out_factory != nullptr && probe_types != nullptr && n_probe_types > 0 && n_probe_output >= 0 &&
                n_build_output >= 0, "invalid arguments");
        auto *base = reinterpret_cast<OperatorFactory *>(hash_builder_factory_addr);
        auto *builder = dynamic_cast<HashBuilderOperatorFactory *>(base);
        Require(builder != nullptr, "hash_builder_factory_addr is not a hash builder factory");
        std::vector<int32_t> po(probe_output_cols, probe_output_cols + n_probe_output);
        std::vector<int32_t> bo(build_output_cols, build_output_cols + n_build_output);
        auto *f = omniruntime::op::LookupOuterJoinOperatorFactory::CreateLookupOuterJoinOperatorFactory(
            ToTypes(probe_types, n_probe_types), po.data(), n_probe_output, bo.data(),
            ToTypes(build_output_types, n_build_output), reinterpret_cast<int64_t>(builder),
            static_cast<omniruntime::op::BuildSide>(build_side));
        *out_factory = static_cast<OperatorFactory *>(f);
    });
}

// ---- join filter expressions
namespace {
namespace ex = omniruntime::expressions;
}

int32_t omg_expr_field(int32_t col, const OmgDataType *type, void **out_expr)
{
    return Guard([&] {
        Require(type != nullptr && out_expr != nullptr && col >= 0, "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::FieldExpr(col, ToType(*type)));
    });
}

int32_t omg_expr_literal_long(int64_t value, const OmgDataType *type, int32_t is_null, void **out_expr)
{
    return Guard([&] {
        Require(type != nullptr && out_expr != nullptr, "invalid arguments");
        auto *l = new ex::LiteralExpr(value, ToType(*type));
        l->isNull = is_null != 0;
        *out_expr = static_cast<ex::Expr *>(l);
    });
}

int32_t omg_expr_literal_double(double value, int32_t is_null, void **out_expr)
{
    return Guard([&] {
        Require(out_expr != nullptr, "invalid arguments");
        auto *l = new ex::LiteralExpr(value, omniruntime::type::DoubleType());
        l->isNull = is_null != 0;
        *out_expr = static_cast<ex::Expr *>(l);
    });
}

int32_t omg_expr_literal_string(const char *bytes, int32_t len, const OmgDataType *type, int32_t is_null,
    void **out_expr)
{
    return Guard([&] {
        Require(type != nullptr && out_expr != nullptr && len >= 0 && (bytes != nullptr || len == 0) &&
                (type->id == omniruntime::type::OMNI_VARCHAR || type->id == omniruntime::type::OMNI_CHAR),
            "invalid arguments");
        auto *l = new ex::LiteralExpr(new std::string(bytes == nullptr ? "" : std::string(bytes, len)), ToType(*type));
        l->isNull = is_null != 0;
        *out_expr = static_cast<ex::Expr *>(l);
    });
}

int32_t omg_expr_func(const char *name, void *const *args, int32_t n_args, const OmgDataType *return_type,
    void **out_expr)
{
    return Guard([&] {
        Require(name != nullptr && return_type != nullptr && out_expr != nullptr && n_args >= 0 &&
                (args != nullptr || n_args == 0),
            "invalid arguments");
        std::vector<ex::Expr *> a(static_cast<size_t>(n_args));
        for (int32_t i = 0; i < n_args; ++i) {
            Require(args[i] != nullptr, "null function argument");
            a[i] = static_cast<ex::Expr *>(args[i]);
        }
        *out_expr = static_cast<ex::Expr *>(new ex::FuncExpr(name, std::move(a), ToType(*return_type)));
    });
}

int32_t omg_expr_binary(int32_t op, void *left, void *right, void **out_expr)
{
    return Guard([&] {
        Require(left != nullptr && right != nullptr && out_expr != nullptr && op >= 0 &&
                op < static_cast<int32_t>(ex::Operator::INVALIDOP),
            "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::BinaryExpr(static_cast<ex::Operator>(op),
            static_cast<ex::Expr *>(left), static_cast<ex::Expr *>(right), omniruntime::type::BooleanType()));
    });
}

int32_t omg_expr_binary_typed(int32_t op, void *left, void *right, const OmgDataType *type, void **out_expr)
{
    return Guard([&] {
        Require(left != nullptr && right != nullptr && out_expr != nullptr && type != nullptr && op >= 0 &&
                op < static_cast<int32_t>(ex::Operator::INVALIDOP),
            "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::BinaryExpr(static_cast<ex::Operator>(op),
            static_cast<ex::Expr *>(left), static_cast<ex::Expr *>(right), ToType(*type)));
    });
}

int32_t omg_expr_unary(int32_t op, void *child, void **out_expr)
{
    return Guard([&] {
        Require(child != nullptr && out_expr != nullptr && op >= 0 &&
                op < static_cast<int32_t>(ex::Operator::INVALIDOP),
            "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::UnaryExpr(static_cast<ex::Operator>(op),
            static_cast<ex::Expr *>(child), omniruntime::type::BooleanType()));
    });
}

int32_t omg_expr_if(void *cond, void *then_expr, void *else_expr, void **out_expr)
{
    return Guard([&] {
        Require(cond != nullptr && then_expr != nullptr && else_expr != nullptr && out_expr != nullptr,
            "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::IfExpr(static_cast<ex::Expr *>(cond),
            static_cast<ex::Expr *>(then_expr), static_cast<ex::Expr *>(else_expr)));
    });
}

int32_t omg_expr_switch(void *const *conds, void *const *results, int32_t n_whens, void *else_expr, void **out_expr)
{
    return Guard([&] {
        Require(conds != nullptr && results != nullptr && n_whens > 0 && else_expr != nullptr && out_expr != nullptr,
            "invalid arguments");
        std::vector<std::pair<ex::Expr *, ex::Expr *>> whens;
        for (int32_t i = 0; i < n_whens; ++i) {
            Require(conds[i] != nullptr && results[i] != nullptr, "null CASE clause");
            whens.emplace_back(static_cast<ex::Expr *>(conds[i]), static_cast<ex::Expr *>(results[i]));
        }
        *out_expr = static_cast<ex::Expr *>(new ex::SwitchExpr(std::move(whens), static_cast<ex::Expr *>(else_expr)));
    });
}

int32_t omg_expr_coalesce(void *value1, void *value2, void **out_expr)
{
    return Guard([&] {
        Require(value1 != nullptr && value2 != nullptr && out_expr != nullptr, "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(
            new ex::CoalesceExpr(static_cast<ex::Expr *>(value1), static_cast<ex::Expr *>(value2)));
    });
}

int32_t omg_expr_in(void *const *args, int32_t n_args, void **out_expr)
{
    return Guard([&] {
        Require(args != nullptr && n_args >= 2 && out_expr != nullptr, "invalid arguments");
        std::vector<ex::Expr *> a(static_cast<size_t>(n_args));
        for (int32_t i = 0; i < n_args; ++i) {
            Require(args[i] != nullptr, "null IN argument");
            a[i] = static_cast<ex::Expr *>(args[i]);
        }
        *out_expr = static_cast<ex::Expr *>(new ex::InExpr(std::move(a)));
    });
}

int32_t omg_expr_between(void *value, void *lower, void *upper, void **out_expr)
{
    return Guard([&] {
        Require(value != nullptr && lower != nullptr && upper != nullptr && out_expr != nullptr, "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::BetweenExpr(static_cast<ex::Expr *>(value),
            static_cast<ex::Expr *>(lower), static_cast<ex::Expr *>(upper)));
    });
}

int32_t omg_expr_is_null(void *child, void **out_expr)
{
    return Guard([&] {
        Require(child != nullptr && out_expr != nullptr, "invalid arguments");
        *out_expr = static_cast<ex::Expr *>(new ex::IsNullExpr(static_cast<ex::Expr *>(child)));
    });
}

int32_t omg_expr_free(void *expr)
{
    delete static_cast<ex::Expr *>(expr);
    return OMG_OK;
}

int32_t omg_lookupjoin_factory_create(const OmgDataType *probe_types, int32_t n_probe_types,
    const int32_t *probe_output_cols, int32_t n_probe_output, const int32_t *probe_hash_cols, int32_t n_probe_hash,
    const int32_t *build_output_cols, int32_t n_build_output, const OmgDataType *build_output_types,
    int64_t hash_builder_factory_addr, const void *filter_expr, int32_t is_shuffle_exchange_build_plan,
    void **out_factory)
{
    return Guard([&] {
        Require(out_factory != nullptr && probe_types != nullptr && n_probe_types > 0, "invalid arguments");
        auto *base = reinterpret_cast<OperatorFactory *>(hash_builder_factory_addr);
        auto *builder = dynamic_cast<HashBuilderOperatorFactory *>(base);
        Require(builder != nullptr, "hash_builder_factory_addr is not a hash builder factory");
        std::vector<int32_t> po(probe_output_cols, probe_output_cols + n_probe_output);
        std::vector<int32_t> ph(probe_hash_cols, probe_hash_cols + n_probe_hash);
        std::vector<int32_t> bo(build_output_cols, build_output_cols + n_build_output);
        auto *f = LookupJoinOperatorFactory::CreateLookupJoinOperatorFactory(ToTypes(probe_types, n_probe_types),
            po.data(), n_probe_output, ph.data(), n_probe_hash, bo.data(), n_build_output,
            ToTypes(build_output_types, n_build_output), reinterpret_cast<int64_t>(builder), filter_expr,
            is_shuffle_exchange_build_plan != 0, nullptr);
        *out_factory = static_cast<OperatorFactory *>(f);
    });
}

int32_t omg_factory_create_operator(void *factory, void **out_op)
{
    return Guard([&] {
        Require(factory != nullptr && out_op != nullptr, "null handle");
        *out_op = static_cast<OperatorFactory *>(factory)->CreateOperator();
    });
}

int32_t omg_factory_destroy(void *factory)
{
    return Guard([&] { delete static_cast<OperatorFactory *>(factory); });
}

// ---- operators
int32_t omg_op_init(void *op)
{
    return Guard([&] { AsOp(op)->Init(); });
}

int32_t omg_op_add_input(void *op, void *batch, int32_t *ret)
{
    return Guard([&] {
        Operator *o = AsOp(op);
        Require(batch != nullptr, "null batch");
        const int32_t r = o->AddInput(static_cast<VectorBatch *>(batch));
        if (ret != nullptr) {
            *ret = r;
        }
    });
}

int32_t omg_op_get_output(void *op, void **out_batch, int32_t *ret)
{
    return Guard([&] {
        Operator *o = AsOp(op);
        Require(out_batch != nullptr, "null output pointer");
        VectorBatch *b = nullptr;
        const int32_t r = o->GetOutput(&b);
        *out_batch = b;
        if (ret != nullptr) {
            *ret = r;
        }
    });
}

int32_t omg_op_add_inputs(void *op, void *const *batches, int32_t n, int32_t *consumed)
{
    if (consumed != nullptr) {
        *consumed = 0;
    }
    return Guard([&] {
        Operator *o = AsOp(op);
        Require(n >= 0 && (n == 0 || batches != nullptr), "null batch array");
        for (int32_t i = 0; i < n; ++i) {
            Require(batches[i] != nullptr, "null batch");
            if (consumed != nullptr) {
                *consumed = i + 1;  // AddInput owns the batch from here on, also when it throws
            }
            o->AddInput(static_cast<VectorBatch *>(batches[i]));
        }
    });
}

int32_t omg_op_get_outputs(void *op, void **out_batches, int32_t max, int32_t *n, int64_t *rows)
{
    if (n != nullptr) {
        *n = 0;
    }
    if (rows != nullptr) {
        *rows = 0;
    }
    return Guard([&] {
        Operator *o = AsOp(op);
        Require(n != nullptr && max >= 0 && (max == 0 || out_batches != nullptr), "null output array");
        while (*n < max) {
            VectorBatch *b = nullptr;
            o->GetOutput(&b);
            if (b == nullptr) {
                break;
            }
            out_batches[(*n)++] = b;
            if (rows != nullptr) {
                *rows += b->GetRowCount();
            }
        }
    });
}

int32_t omg_op_get_sizing_log(void *op, int64_t *out, int32_t n, int32_t *written)
{
    return Guard([&] {
        auto *agg = dynamic_cast<HashAggregationOperator *>(AsOp(op));
        Require(agg != nullptr, "not a HashAggregation operator");
        Require(out != nullptr && n >= 0 && written != nullptr, "null output");
        *written = agg->GetSizingLog(out, n);
    });
}

// ---- learned sizing model
namespace {
omg::SizingModel *AsSizer(void *m)
{
    Require(m != nullptr, "null model");
    return static_cast<omg::SizingModel *>(m);
}
}  // namespace

int32_t omg_sizer_create(const int32_t *dims, int32_t n_dims, uint64_t seed, void **out_model)
{
    return Guard([&] {
        Require(dims != nullptr && n_dims >= 2 && n_dims <= 16 && out_model != nullptr, "bad model dims");
        *out_model = new omg::SizingModel(std::vector<int32_t>(dims, dims + n_dims), seed);
    });
}

int32_t omg_sizer_destroy(void *model)
{
    return Guard([&] { delete static_cast<omg::SizingModel *>(model); });
}

int32_t omg_sizer_num_params(void *model, int64_t *n_params)
{
    return Guard([&] {
        Require(n_params != nullptr, "null output");
        *n_params = AsSizer(model)->NumParams();
    });
}

int32_t omg_sizer_get_params(void *model, float *params, int64_t n_params)
{
    return Guard([&] {
        omg::SizingModel *m = AsSizer(model);
        Require(params != nullptr && n_params == m->NumParams(), "parameter count mismatch");
        m->GetParams(params);
    });
}

int32_t omg_sizer_set_params(void *model, const float *params, int64_t n_params)
{
    return Guard([&] {
        omg::SizingModel *m = AsSizer(model);
        Require(params != nullptr && n_params == m->NumParams(), "parameter count mismatch");
        m->SetParams(params);
    });
}

int32_t omg_sizer_predict(void *model, const float *X, int32_t n, float *Y)
{
    return Guard([&] {
        Require(n >= 0 && (n == 0 || (X != nullptr && Y != nullptr)), "null array");
        AsSizer(model)->Predict(X, n, Y);
    });
}

int32_t omg_sizer_gradients(void *model, const float *X, const float *T, int32_t n, float *grad, float *loss)
{
    return Guard([&] {
        Require(n > 0 && X != nullptr && T != nullptr && grad != nullptr, "null array");
        const float l = AsSizer(model)->Gradients(X, T, n, grad);
        if (loss != nullptr) {
            *loss = l;
        }
    });
}

int32_t omg_sizer_train(void *model, const float *X, const float *T, int32_t n, int32_t epochs, float lr,
    float *loss)
{
    return Guard([&] {
        Require(n > 0 && X != nullptr && T != nullptr && epochs > 0 && lr > 0.f, "bad training arguments");
        const float l = AsSizer(model)->Train(X, T, n, epochs, lr);
        if (loss != nullptr) {
            *loss = l;
        }
    });
}

int32_t omg_sizer_features(const int64_t *sizing_log, int32_t n_log, float *features)
{
    return Guard([&] {
        Require(sizing_log != nullptr && n_log >= 1 + omg::kSketchStats && features != nullptr, "bad sizing log");
        omg::SizerFeatures(sizing_log, features);
    });
}

int32_t omg_sizer_target(const int64_t *sizing_log, int32_t n_log, int64_t groups, float *target)
{
    return Guard([&] {
        Require(sizing_log != nullptr && n_log >= 1 + omg::kSketchStats && target != nullptr, "bad sizing log");
        *target = omg::SizerTarget(sizing_log, groups);
    });
}

int32_t omg_sizer_estimate(const int64_t *sizing_log, int32_t n_log, float y, int64_t *estimate)
{
    return Guard([&] {
        Require(sizing_log != nullptr && n_log >= 1 + omg::kSketchStats && estimate != nullptr, "bad sizing log");
        *estimate = static_cast<int64_t>(omg::SizerEstimate(sizing_log, y));
    });
}

int32_t omg_hashagg_factory_set_sizer(void *factory, void *model)
{
    return Guard([&] {
        auto *f = dynamic_cast<HashAggregationOperatorFactory *>(static_cast<OperatorFactory *>(factory));
        Require(f != nullptr, "not a HashAggregation factory");
        if (model != nullptr) {
            Require(AsSizer(model)->Dims()[0] == omg::kSizerFeatures, "model input width must be 12");
        }
        f->SetSizer(static_cast<omg::SizingModel *>(model));
    });
}

// ---- batched aggregation
namespace {
struct AggBatchHandle {
    std::unique_ptr<omniruntime::op::BatchedAggregation> agg;
    std::vector<VectorBatch *> pending;
    std::vector<int32_t> pendingTask;
    size_t next = 0;
    void DropPending()
    {
        for (size_t i = next; i < pending.size(); ++i) {
            VectorHelper::FreeVecBatch(pending[i]);
        }
        pending.clear();
        pendingTask.clear();
        next = 0;
    }
};
AggBatchHandle *AsAggBatch(void *b)
{
    Require(b != nullptr, "null batch handle");
    return static_cast<AggBatchHandle *>(b);
}
}  // namespace

int32_t omg_agg_batch_create(void *factory, void *const *task_batches, int32_t n_tasks, void *sizer, int32_t flags,
    void **out_batch)
{
    return Guard([&] {
        auto *f = dynamic_cast<HashAggregationOperatorFactory *>(static_cast<OperatorFactory *>(factory));
        Require(f != nullptr, "not a HashAggregation factory");
        Require(n_tasks > 0 && task_batches != nullptr && out_batch != nullptr, "no tasks");
        std::vector<VectorBatch *> tasks(n_tasks);
        for (int32_t i = 0; i < n_tasks; ++i) {
            tasks[i] = static_cast<VectorBatch *>(task_batches[i]);
        }
        auto h = std::make_unique<AggBatchHandle>();
        h->agg.reset(new omniruntime::op::BatchedAggregation(*f, tasks, static_cast<omg::SizingModel *>(sizer), flags));
        *out_batch = h.release();
    });
}

int32_t omg_agg_batch_run(void *batch, void *stream)
{
    return Guard([&] {
        AggBatchHandle *h = AsAggBatch(batch);
        h->DropPending();
        h->agg->Run(stream);
        h->agg->Outputs(h->pending, h->pendingTask);
    });
}

int32_t omg_agg_batch_outputs(void *batch, void **out_batches, int32_t *task_of, int32_t max, int32_t *n)
{
    return Guard([&] {
        AggBatchHandle *h = AsAggBatch(batch);
        Require(n != nullptr && max >= 0 && (max == 0 || out_batches != nullptr), "null output array");
        int32_t k = 0;
        while (k < max && h->next < h->pending.size()) {
            out_batches[k] = h->pending[h->next];
            if (task_of != nullptr) {
                task_of[k] = h->pendingTask[h->next];
            }
            ++k;
            ++h->next;
        }
        *n = k;
    });
}

int32_t omg_agg_batch_info(void *batch, int64_t *out, int32_t n, int32_t *written)
{
    return Guard([&] {
        Require(out != nullptr && written != nullptr && n >= 0, "null output");
        const std::vector<int64_t> v = AsAggBatch(batch)->agg->Info();
        const int32_t m = std::min<int32_t>(n, static_cast<int32_t>(v.size()));
        std::copy(v.begin(), v.begin() + m, out);
        *written = m;
    });
}

int32_t omg_agg_batch_sizing_logs(void *batch, int64_t *out, int64_t n, int64_t *written)
{
    return Guard([&] {
        Require(out != nullptr && written != nullptr && n >= 0, "null output");
        const std::vector<int64_t> v = AsAggBatch(batch)->agg->SizingLogs();
        const int64_t m = std::min<int64_t>(n, static_cast<int64_t>(v.size()));
        std::copy(v.begin(), v.begin() + m, out);
        *written = m;
    });
}

int32_t omg_agg_batch_destroy(void *batch)
{
    return Guard([&] {
        if (batch == nullptr) {
            return;
        }
        auto *h = static_cast<AggBatchHandle *>(batch);
        h->DropPending();
        delete h;
    });
}

int32_t omg_op_set_join_strategy(void *op, int32_t strategy, int32_t bits, const int64_t *splits, int32_t n_splits)
{
    return Guard([&] {
        auto *j = dynamic_cast<omniruntime::op::LookupJoinOperator *>(AsOp(op));
        Require(j != nullptr, "not a LookupJoin operator");
        j->SetJoinStrategy(strategy, bits, splits, n_splits);
    });
}

int32_t omg_op_join_strategy(void *op, int32_t *strategy)
{
    return Guard([&] {
        auto *j = dynamic_cast<omniruntime::op::LookupJoinOperator *>(AsOp(op));
        Require(j != nullptr && strategy != nullptr, "not a LookupJoin operator");
        *strategy = j->JoinStrategy();
    });
}

int32_t omg_join_learn_splits(const int64_t *sample, int64_t n, int32_t bits, int32_t epochs, uint64_t seed,
    int64_t *splits)
{
    return Guard([&] {
        Require(sample != nullptr && splits != nullptr, "null array");
        omg::LearnRangeSplits(sample, n, bits, epochs, seed, splits);
    });
}

int32_t omg_join_quantile_splits(const int64_t *sample, int64_t n, int32_t bits, int64_t *splits)
{
    return Guard([&] {
        Require(sample != nullptr && splits != nullptr, "null array");
        omg::QuantileSplits(sample, n, bits, splits);
    });
}

int32_t omg_batches_fingerprint(void *const *batches, int32_t n, uint64_t *out)
{
    return Guard([&] {
        Require(out != nullptr && n >= 0 && (n == 0 || batches != nullptr), "null array");
        out[0] = out[1] = out[2] = 0;
        if (n == 0) {
            return;
        }
        omg::RequireDevice();
        std::vector<VectorBatch *> list(n);
        for (int32_t i = 0; i < n; ++i) {
            list[i] = static_cast<VectorBatch *>(batches[i]);
            Require(list[i] != nullptr, "null batch");
        }
        const int32_t nCols = list[0]->GetVectorCount();
        Require(nCols <= omg::kMaxInputs, "too many columns");
        std::vector<int32_t> cols(nCols), widths(nCols);
        for (int32_t c = 0; c < nCols; ++c) {
            cols[c] = c;
            widths[c] = list[0]->Get(c)->GetWidth();
        }
        cudaStream_t s = omg::AcquirePooledStream();
        try {
            omg::BatchTable bt;
            bt.Build(list, cols);
            bt.Upload(s);
            omg::DevArray<int32_t> w(nCols, s);
            omg::DevArray<unsigned long long> fp(3, s);
            omg::CudaCheck(cudaMemcpyAsync(w.Get(), widths.data(), sizeof(int32_t) * nCols, cudaMemcpyHostToDevice, s),
                "upload widths");
            omg::CudaCheck(omg::LaunchFingerprint(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(), nCols, w.Get(),
                               fp.Get(), s),
                "fingerprint");
            unsigned long long h[3];
            omg::CudaCheck(cudaMemcpyAsync(h, fp.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read fingerprint");
            omg::CudaCheck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            out[0] = h[0];
            out[1] = h[1];
            out[2] = h[2];
        } catch (...) {
            omg::ReleasePooledStream(s);
            throw;
        }
        omg::ReleasePooledStream(s);
    });
}

int32_t omg_batch_free_many(void *const *batches, int32_t n)
{
    return Guard([&] {
        Require(n >= 0 && (n == 0 || batches != nullptr), "null batch array");
        for (int32_t i = 0; i < n; ++i) {
            if (batches[i] != nullptr) {
                VectorHelper::FreeVecBatch(static_cast<VectorBatch *>(batches[i]));
            }
        }
    });
}

int32_t omg_op_status(void *op) { return op ? static_cast<int32_t>(static_cast<Operator *>(op)->GetStatus()) : -1; }

int32_t omg_op_no_more_input(void *op)
{
    return Guard([&] { AsOp(op)->noMoreInput(); });
}

int32_t omg_op_set_no_more_input(void *op, int32_t no_more_input)
{
    return Guard([&] { AsOp(op)->setNoMoreInput(no_more_input != 0); });
}

int32_t omg_op_needs_input(void *op) { return op ? (static_cast<Operator *>(op)->needsInput() ? 1 : 0) : -1; }

int32_t omg_op_is_blocked(void *op)
{
    if (op == nullptr) {
        return -1;
    }
    return static_cast<Operator *>(op)->IsBlocked() == omniruntime::op::BlockingReason::kNotBlocked ? 0 : 1;
}

int64_t omg_op_hashmap_unique_keys(void *op)
{
    return op ? static_cast<int64_t>(static_cast<Operator *>(op)->GetHashMapUniqueKeys()) : -1;
}

int32_t omg_op_align_schema(void *op, void *batch, void **out)
{
    return Guard([&] {
        if (out != nullptr) {
            *out = nullptr;
        }
        auto *b = static_cast<VectorBatch *>(batch);
        if (op == nullptr || b == nullptr || out == nullptr) {
            if (b != nullptr) {
                omniruntime::vec::VectorHelper::FreeVecBatch(b);
            }
            Require(false, "null handle");
        }
        *out = AsOp(op)->AlignSchema(b);
    });
}

int32_t omg_op_close(void *op)
{
    return Guard([&] { AsOp(op)->Close(); });
}

int32_t omg_op_delete(void *op)
{
    return Guard([&] {
        if (op != nullptr) {
            Operator::DeleteOperator(static_cast<Operator *>(op));
        }
    });
}

int32_t omg_op_set_stream(void *op, void *stream)
{
    return Guard([&] { AsOp(op)->SetStream(stream); });
}

int32_t omg_op_set_device_output(void *op, int32_t on)
{
    return Guard([&] { AsOp(op)->SetDeviceOutput(on != 0); });
}

int32_t omg_op_set_agg_strategy(void *op, int32_t strategy, int64_t capacity_hint)
{
    return Guard([&] {
        auto *a = dynamic_cast<HashAggregationOperator *>(AsOp(op));
        Require(a != nullptr, "not a hash aggregation operator");
        Require(strategy >= OMG_AGG_STRATEGY_AUTO && strategy <= OMG_AGG_STRATEGY_PARTITIONED, "unknown strategy");
        a->SetStrategy(strategy, capacity_hint);
    });
}

int32_t omg_op_set_agg_sizing(void *op, int32_t mode)
{
    return Guard([&] {
        auto *a = dynamic_cast<HashAggregationOperator *>(AsOp(op));
        Require(a != nullptr, "not a hash aggregation operator");
        Require(mode == OMG_AGG_SIZING_SAMPLE || mode == OMG_AGG_SIZING_HLL, "unknown sizing mode");
        a->SetSizing(mode);
    });
}

int32_t omg_op_set_spill(void *op, int32_t enabled, int64_t device_budget_bytes)
{
    return Guard([&] {
        auto *a = dynamic_cast<HashAggregationOperator *>(AsOp(op));
        Require(a != nullptr, "not a hash aggregation operator");
        Require(device_budget_bytes >= 0, "invalid budget");
        a->SetSpill(enabled != 0, static_cast<uint64_t>(device_budget_bytes));
    });
}

int64_t omg_op_spilled_bytes(void *op)
{
    return op ? static_cast<int64_t>(AsOp(op)->GetSpilledBytes()) : -1;
}

int32_t omg_hashagg_run_noalloc(void *factory, const void *const *d_cols, const uint8_t *const *d_nulls,
    int32_t n_cols, int64_t n_rows, void *const *d_out_values, uint8_t *const *d_out_nulls, int32_t n_out,
    int64_t max_groups, int64_t *num_groups, void *stream)
{
    ClearError();
    auto *f = dynamic_cast<HashAggregationOperatorFactory *>(static_cast<OperatorFactory *>(factory));
    if (f == nullptr) {
        SetError("not a hash aggregation factory");
        return OMG_ERR_INVALID_ARG;
    }
    const auto &ap = f->Plan();
    if (!ap.dictInputs.empty() || !ap.varlenInputs.empty()) {
        // String columns need the operator's per-call string dictionary (device allocations).
        SetError("VARCHAR/CHAR columns are not supported by the allocation-free entry point");
        return OMG_ERR_UNSUPPORTED;
    }
    if (std::any_of(ap.inputMasks.begin(), ap.inputMasks.end(), [](int32_t m) { return m != -1; })) {
        // A mask turns into a per-call NULL bitmap of the masked inputs (a device allocation).
        SetError("aggregation mask columns are not supported by the allocation-free entry point");
        return OMG_ERR_UNSUPPORTED;
    }
    if (!omg::DeviceAvailable()) {
        SetError("no CUDA device is available");
        return OMG_ERR_NO_DEVICE;
    }
    for (int32_t c : ap.outContainer) {
        if (c > 0) {
            SetError("container-vector outputs are not supported by the allocation-free entry point");
            return OMG_ERR_UNSUPPORTED;
        }
    }
    omg::NoAllocPlan np;
    np.nInputs = static_cast<int32_t>(ap.inputCols.size());
    for (int32_t i = 0; i < np.nInputs; ++i) {
        if (ap.inputCols[i] >= omg::kFieldRefBase) {
            SetError("container-vector inputs are not supported by the allocation-free entry point");
            return OMG_ERR_UNSUPPORTED;
        }
        np.inputCols[i] = ap.inputCols[i];
    }
    np.key = ap.key;
    np.nAccs = static_cast<int32_t>(ap.accs.size());
    for (int32_t i = 0; i < np.nAccs; ++i) {
        np.accs[i] = ap.accs[i];
    }
    np.nRegInputs = static_cast<int32_t>(ap.regInput.size());
    for (int32_t i = 0; i < np.nRegInputs; ++i) {
        np.regInput[i] = ap.regInput[i];
        np.regWidth[i] = ap.regWidth[i];
    }
    np.stateWords = ap.stateWords;
    np.keyWords = ap.keyWords;
    np.slotWords = ap.slotWords;
    np.nOut = static_cast<int32_t>(ap.outs.size());
    for (int32_t i = 0; i < np.nOut; ++i) {
        np.outs[i] = ap.outs[i];
    }
    np.overflowAsNull = ap.overflowAsNull;
    np.smemSlots = ap.smemSlots;
    np.waitBudget = omg::WaitBudget();
    const omg::NoAllocStatus st = omg::RunAggNoAlloc(np, d_cols, d_nulls, n_cols, n_rows, d_out_values, d_out_nulls,
        n_out, max_groups, num_groups, static_cast<cudaStream_t>(stream));
    if (st.code != 0) {
        SetError(st.message);
    }
    return st.code;
}

int32_t omg_op_get_counters(void *op, int64_t *out, int32_t n)
{
    return Guard([&] {
        Require(out != nullptr && n >= 0, "invalid arguments");
        const auto &c = AsOp(op)->Counters();
        for (int32_t i = 0; i < n; ++i) {
            out[i] = i < static_cast<int32_t>(c.size()) ? c[i] : 0;
        }
    });
}

}  // extern "C"
