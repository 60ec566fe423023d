/*
 * omniop_gb300.h -- C ABI of the GB300-native hash aggregation / hash join operators.
 *
 * Every entry point is plain C: opaque handles, plain pointers and sizes, an int32
 * status code (OMG_OK == 0) and a thread-local error message (omg_last_error()).
 * No C++ exception, torch type or CUDA type crosses this boundary; CUDA streams are
 * passed as `void*` (a cudaStream_t) and may be NULL for the operator's own stream.
 *
 * The operator API mirrors OmniOperator's C++ operator surface, which its JNI layer
 * binds (bindings/java/src/main/cpp/src/jni_operator.cpp:159-215 and
 * jni_operator_factory.cpp:177-236,585-606,620-).  Each declaration below names
 * the reference interface it replaces.
 *
 * Memory model.  Vectors are either HOST vectors (page-locked host memory the GPU
 * reads directly, the OmniVec layout: flat values + LSB-first null bitmap where a
 * set bit means NULL) or DEVICE vectors (HBM; owned, or a non-owning view of memory
 * the caller owns).  AddInput accepts either; GetOutput returns host vectors unless
 * the operator was switched to device output.
 */
#ifndef OMNIOP_GB300_H
#define OMNIOP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define OMG_OK 0
#define OMG_ERR_INVALID_ARG (-1)
#define OMG_ERR_UNSUPPORTED (-2)
#define OMG_ERR_CUDA (-3)
#define OMG_ERR_OOM (-4)
#define OMG_ERR_OVERFLOW (-5)      /* sum overflow with overflow-as-null off (OmniException) */
#define OMG_ERR_STATE (-6)         /* call not valid in the operator's current state */
#define OMG_ERR_TIMEOUT (-7)       /* a bounded device-side wait ran out */
#define OMG_ERR_NO_DEVICE (-8)     /* no CUDA device: compute entry points refuse to run */
#define OMG_ERR_INTERNAL (-9)

/* Data type ids: same numbering as type/data_type.h:40-74 (DataTypeId). */
#define OMG_TYPE_INT 1
#define OMG_TYPE_LONG 2
#define OMG_TYPE_DOUBLE 3
#define OMG_TYPE_BOOLEAN 4
#define OMG_TYPE_SHORT 5
#define OMG_TYPE_DECIMAL64 6
#define OMG_TYPE_DECIMAL128 7
#define OMG_TYPE_DATE32 8
#define OMG_TYPE_DATE64 9
#define OMG_TYPE_TIMESTAMP 12
#define OMG_TYPE_BYTE 18
#define OMG_TYPE_FLOAT 19
#define OMG_TYPE_FIXEDBINARY 40 /* fixed-width byte string (width bytes per row); no reference id */

/* Aggregate function ids: same numbering as operator/util/function_type.h:11-27. */
#define OMG_AGG_SUM 0
#define OMG_AGG_COUNT_COLUMN 1
#define OMG_AGG_COUNT_ALL 2
#define OMG_AGG_AVG 3
#define OMG_AGG_MAX 5
#define OMG_AGG_MIN 6

/* Join types: plannode/planNode.h:406-414.  Only INNER is built. */
#define OMG_JOIN_INNER 0

/* Operator status: operator/status.h:9-13. */
#define OMG_STATUS_NORMAL 0
#define OMG_STATUS_FINISHED 1
#define OMG_STATUS_ERROR (-1)

/* Policy knobs: util/policy.h:160-186 (SupportContainerVecRule) and
 * operator/config/operator_config.h:168-190 (OverflowConfig). */
#define OMG_POLICY_SPARK 0   /* SupportContainerVecRule::NOT_SUPPORT (reference default) */
#define OMG_POLICY_GENERIC 1 /* SupportContainerVecRule::SUPPORT */

/* Aggregation strategy hints (GB300-specific; results never depend on them). */
#define OMG_AGG_STRATEGY_AUTO 0
#define OMG_AGG_STRATEGY_SMEM 1   /* shared-memory pre-aggregation, global overflow */
#define OMG_AGG_STRATEGY_GLOBAL 2 /* global open-addressing table only */
#define OMG_AGG_STRATEGY_PARTITIONED 3 /* hash partitions, a shared-memory table per partition */

/* A column type: id plus decimal precision/scale (or FIXEDBINARY width). */
typedef struct OmgDataType {
    int32_t id;
    int32_t precision;
    int32_t scale;
    int32_t width;
} OmgDataType;

/* ---- errors / runtime ------------------------------------------------------------- */
/* Thread-local message of the last failing call on this thread ("" if none). */
const char *omg_last_error(void);
/* Library version string. */
const char *omg_version(void);
/* 1 if a CUDA device is usable by this process, else 0. */
int32_t omg_device_available(void);
/* Set the policy used by factories created afterwards (ConfigUtil::SetSupportContainerVecRule,
 * util/config_util.h).  OMG_POLICY_SPARK is the default. */
int32_t omg_config_set_policy(int32_t policy);
int32_t omg_config_get_policy(void);
/* substr policies (util/policy.h:70-100, ConfigUtil::SetNegativeStartIndexOutOfBoundsRule and
 * SetZeroStartIndexSupportRule): negative_rule 0 EMPTY_STRING, 1 INTERCEPT_FROM_BEYOND (default);
 * zero_rule 0 IS_NOT_SUPPORT, 1 IS_SUPPORT (default).  Read by join factories created afterwards. */
int32_t omg_config_set_substr_rules(int32_t negative_rule, int32_t zero_rule);
int32_t omg_config_get_substr_rules(int32_t *negative_rule, int32_t *zero_rule);
/* Fault injection on the host: the next `n` device allocations of this library fail
 * with OMG_ERR_OOM (0 disables).  Used by the tests; never touches the GPU. */
int32_t omg_debug_fail_next_allocs(int32_t n);
/* Device-side bounded-wait budget in clock64 ticks (0 = library default). */
int32_t omg_debug_set_wait_budget(int64_t ticks);
/* Inner probes on a bitmap ARRAY table that write pinned host output: 1 (default) = the
 * group-staged kernel (whole-line output runs over the CPU-GPU link), 0 = the per-warp bitmap
 * kernel (always used for HBM output).  Both give the same rows; for tests and measurements.
 * No reference counterpart. */
int32_t omg_debug_set_staged_probe(int32_t on);
/* Inner probes on a bitmap ARRAY table from device-resident keys to HBM output: 0 (default) =
 * the per-lane bitmap kernel, 1 = the bulk-copy kernel with keys moved into shared memory by
 * cp.async.bulk, 2 = the same with output runs stored back by cp.async.bulk.  All give the same
 * rows; for tests and measurements.  No reference counterpart. */
int32_t omg_debug_set_bulk_probe(int32_t mode);
/* Which probe kernel the latest probe launch in this process started: 1 multi-column keys or
 * filters, 2 general, 3 fast (unique table, register outputs), 4 bitmap with per-lane loads
 * and stores, 5 group-staged (pinned host output), 6 bulk-copy; 0 none yet.  For tests and
 * measurements.  No reference counterpart. */
int32_t omg_debug_last_probe_kernel(void);
/* Train sizing and CDF models of two hidden layers (input <= 16, hidden widths multiples of 4 up
 * to 64) with the fused kernel, all epochs in one cooperative launch (1, default), or layer by
 * layer with one launch per layer and step (0).  For tests and measurements.  No reference
 * counterpart. */
int32_t omg_debug_set_fused_training(int32_t on);
/* Staged rows at which a HashAggregation operator aggregates its queued batches before
 * GetOutput (0 = library default, 2^28).  Process-wide; lets tests run many batch sets
 * through one operator. */
int32_t omg_debug_set_agg_flush_rows(int64_t rows);
/* Queued probe rows at which a pipelined LookupJoin operator (SetNoMoreInput(false) callers)
 * hands a chunk to its worker thread (0 = library default, 2^22).  Process-wide; lets tests run
 * the worker pipeline on small inputs. */
int32_t omg_debug_set_probe_chunk_rows(int64_t rows);

/* ---- OmniVec: vectors and batches -------------------------------------------------- */
/* New flat host vector (VectorHelper::CreateFlatVector, vector/vector_helper.h).
 * Values are zeroed, no nulls.  FIXEDBINARY needs omg_vec_new_fixed. */
int32_t omg_vec_new(int32_t type_id, int32_t size, void **out_vec);
int32_t omg_vec_new_fixed(int32_t width, int32_t size, void **out_vec);
/* New host VARCHAR (15) or CHAR (16) vector: size + 1 int32 offsets (zeroed) into a character
 * buffer of `data_bytes` bytes; value i is bytes [offsets[i], offsets[i + 1]) -- the
 * LargeStringContainer layout (vector/vector.h, vector/large_string_container.h). */
int32_t omg_vec_new_varchar(int32_t type_id, int32_t size, int64_t data_bytes, void **out_vec);
/* VARCHAR/CHAR accessors: the offsets array (NULL for fixed-width vectors; omg_vec_values is
 * the character buffer) and the character buffer's size in bytes. */
int32_t *omg_vec_offsets(void *vec);
int64_t omg_vec_data_bytes(void *vec);
/* New flat device vector (HBM, owned by the vector). */
int32_t omg_vec_new_device(int32_t type_id, int32_t width, int32_t size, void **out_vec);
/* Non-owning device view over caller memory.  `nulls` may be NULL (no nulls); when given
 * it is an LSB-first bitmap, set bit = NULL, of ceil(size/8) bytes at least. */
int32_t omg_vec_wrap_device(int32_t type_id, int32_t width, int32_t size, void *values, void *nulls,
    void **out_vec);
/* Delete a vector that is not owned by a batch. */
int32_t omg_vec_free(void *vec);
/* Dictionary-encoded host vector (VectorHelper::CreateDictionaryVector,
 * core/src/vector/vector_helper.h:381-420): row i is row ids[i] of the flat vector `dictionary`
 * (host or device), whose buffers the new vector shares (the dictionary handle stays the caller's
 * and may be freed).  A row is NULL when its dictionary row is.  Ids outside
 * [0, omg_vec_size(dictionary)) are refused with OMG_ERR_INVALID.  Operators flatten such
 * vectors on the device when they take a batch. */
int32_t omg_vec_new_dictionary(const int32_t *ids, int32_t size, void *dictionary, void **out_vec);
/* Vector encoding (BaseVector::GetEncoding, vector/vector.h:107): 0 flat, 1 dictionary,
 * 2 container (operator/aggregation/container_vector.h: a partial AVG's (double sum, long count)
 * under the container-vector policy; type id OMNI_CONTAINER, 17). */
int32_t omg_vec_encoding(void *vec);
/* Container vectors: the number of fields (0 for other vectors) and field i, a flat vector owned
 * by the container (borrowed: do not free it). */
int32_t omg_vec_num_fields(void *vec);
void *omg_vec_field(void *vec, int32_t i);
/* Raw accessors (unsafe/unsafe_vector.h:19-48).  Pointers are host or device
 * addresses according to omg_vec_is_device. */
void *omg_vec_values(void *vec);
uint8_t *omg_vec_nulls(void *vec);
int32_t omg_vec_size(void *vec);
int32_t omg_vec_type(void *vec);
int32_t omg_vec_width(void *vec);
int32_t omg_vec_is_device(void *vec);
/* BaseVector::HasNull / SetNullFlag (vector/vector.h:45-). */
int32_t omg_vec_has_null(void *vec);
int32_t omg_vec_set_null_flag(void *vec, int32_t has_null);

/* VectorBatch (vector/vector_batch.h:10-66). */
int32_t omg_batch_new(int32_t row_count, void **out_batch);
int32_t omg_batch_append(void *batch, void *vec); /* batch takes ownership of vec */
void *omg_batch_get(void *batch, int32_t index);
int32_t omg_batch_row_count(void *batch);
int32_t omg_batch_vector_count(void *batch);
/* VectorHelper::FreeVecBatch: frees the batch and all its vectors. */
int32_t omg_batch_free(void *batch);
/* Copy a batch between host and device residency (new batch, caller owns it). */
int32_t omg_batch_to_device(void *batch, void **out_batch);
int32_t omg_batch_to_host(void *batch, void **out_batch);

/* ---- factories ---------------------------------------------------------------------- */
/* HashAggregationOperatorFactory(groupByCol, groupInputTypes, aggsCols, aggInputTypes,
 *     aggOutputTypes, aggFuncTypes, maskColsVector, inputRaws, outputPartials, overflowAsNull)
 *   -- operator/aggregation/group_aggregation.h:217-249; JNI createHashAggregationOperatorFactory
 *   (jni_operator_factory.cpp:177-236).
 * Aggregator i reads the columns agg_cols[agg_col_offsets[i] .. agg_col_offsets[i+1]) whose
 * types are agg_input_types at the same positions; its output types are
 * agg_output_types[agg_out_offsets[i] .. agg_out_offsets[i+1]).  mask_cols[i] >= 0 names a
 * BOOLEAN column: aggregator i then sees only the rows where that column is TRUE (NULL counts
 * as FALSE; every row still creates its group), as MaskColAggregator does
 * (aggregator/mask_column_assistant_aggregator.h:44-53); -1 means no mask.  input_raws[i] = 0
 * reads partial results and output_partials[i] = 1 emits them (two-stage aggregation). */
int32_t omg_hashagg_factory_create(const uint32_t *group_cols, const OmgDataType *group_types,
    int32_t n_group, const uint32_t *agg_func_types, int32_t n_agg, const int32_t *agg_col_offsets,
    const uint32_t *agg_cols, const OmgDataType *agg_input_types, const int32_t *agg_out_offsets,
    const OmgDataType *agg_output_types, const int32_t *mask_cols, const uint8_t *input_raws,
    const uint8_t *output_partials, int32_t overflow_as_null, void **out_factory);

/* HashBuilderOperatorFactory::CreateHashBuilderOperatorFactory(joinType, buildTypes,
 *     buildHashCols, buildHashColsCount, operatorCount) -- operator/join/hash_builder.h:28-29.
 * join_type: OMNI_JOIN_TYPE_* (inner 0, left 1, right 2, full 3, left semi 4, left anti 5,
 * existence 6); 1 to 4 key columns of fixed width (probe key columns of the same widths). */
int32_t omg_hashbuilder_factory_create(int32_t join_type, const OmgDataType *build_types,
    int32_t n_build_types, const int32_t *build_hash_cols, int32_t n_hash_cols, int32_t operator_count,
    void **out_factory);

/* CreateHashBuilderOperatorFactory(joinType, buildSide, buildTypes, buildHashCols,
 *     buildHashColsCount, operatorCount) -- operator/join/hash_builder.h:30-31.
 * build_side: OMNI_BUILD_UNKNOWN 0, LEFT 1, RIGHT 2 (plannode/planNode.h:29-33).  A left (right)
 * join built on its left (right) input keeps its unmatched build rows, which a
 * LookupOuterJoin operator emits after the probes; with build side LEFT every output batch
 * lists the build columns first. */
int32_t omg_hashbuilder_factory_create_side(int32_t join_type, int32_t build_side,
    const OmgDataType *build_types, int32_t n_build_types, const int32_t *build_hash_cols, int32_t n_hash_cols,
    int32_t operator_count, void **out_factory);

/* LookupOuterJoinOperatorFactory::CreateLookupOuterJoinOperatorFactory(probeTypes,
 *     probeOutputCols, probeOutputColsCount, buildOutputCols, buildOutputTypes,
 *     hashBuilderFactoryAddr, buildSide) -- operator/join/lookup_outer_join.h:28-33.
 * For full joins and build-side outer joins: its operator's GetOutput emits the build rows no
 * probe matched (NULL probe columns), once every probe operator has drained. */
int32_t omg_lookupouterjoin_factory_create(const OmgDataType *probe_types, int32_t n_probe_types,
    const int32_t *probe_output_cols, int32_t n_probe_output, const int32_t *build_output_cols,
    int32_t n_build_output, const OmgDataType *build_output_types, int64_t hash_builder_factory_addr,
    int32_t build_side, void **out_factory);

/* LookupJoinOperatorFactory::CreateLookupJoinOperatorFactory(probeTypes, probeOutputCols, n,
 *     probeHashCols, n, buildOutputCols, n, buildOutputTypes, hashBuilderFactoryAddr, filterExpr,
 *     isShuffleExchangeBuildPlan, overflowConfig) -- operator/join/lookup_join.h:148-152.
 * `filter_expr` must be NULL (join filters are not built). */
int32_t omg_lookupjoin_factory_create(const OmgDataType *probe_types, int32_t n_probe_types,
    const int32_t *probe_output_cols, int32_t n_probe_output, const int32_t *probe_hash_cols,
    int32_t n_probe_hash, const int32_t *build_output_cols, int32_t n_build_output,
    const OmgDataType *build_output_types, int64_t hash_builder_factory_addr, const void *filter_expr,
    int32_t is_shuffle_exchange_build_plan, void **out_factory);

/* ---- join filter expressions (core/src/expression/expressions.h:22-62) -------------
 * Trees of FieldExpr / LiteralExpr / BinaryExpr / UnaryExpr / IsNullExpr nodes for the
 * filter_expr of omg_lookupjoin_factory_create; a field is a column of the joined row (probe
 * columns first, then build columns).  Binary, unary and is-null nodes take ownership of their
 * children; free the root with omg_expr_free (the factory compiles the tree and keeps no pointer
 * into it).  Operator codes follow expressions::Operator: 0 EQ, 1 NEQ, 2 LT, 3 LTE, 4 GT, 5 GTE,
 * 6 AND, 7 OR, 8 NOT, 9 ADD, 10 SUB, 11 MUL, 12 DIV, 13 MOD, 14 TRY_ADD, 15 TRY_SUB, 16 TRY_MUL,
 * 17 TRY_DIV.  The GB300 join runs comparisons, AND, OR, NOT, IS NULL and arithmetic (with the
 * reference's math-function semantics: integers wrap at the node's INT or LONG width, DIV/MOD by
 * zero and TRY_* overflow give NULL) over integer-like and DOUBLE columns and literals, and
 * comparisons of VARCHAR/CHAR columns, literals and substr results (byte-wise unsigned, a
 * proper prefix first: codegen/functions/stringfunctions.cpp StrCompare), IF, CASE, COALESCE,
 * IN and BETWEEN; other trees (other functions, a filter that does not return BOOLEAN) are
 * refused by the factory with OMG_ERR_UNSUPPORTED, as the reference refuses what its code
 * generator cannot compile. */
int32_t omg_expr_field(int32_t col, const OmgDataType *type, void **out_expr);
int32_t omg_expr_literal_long(int64_t value, const OmgDataType *type, int32_t is_null, void **out_expr);
int32_t omg_expr_literal_double(double value, int32_t is_null, void **out_expr);
/* LiteralExpr(std::string *, VarcharType/CharType): `len` bytes at `bytes` (copied). */
int32_t omg_expr_literal_string(const char *bytes, int32_t len, const OmgDataType *type, int32_t is_null,
    void **out_expr);
/* FuncExpr(name, args, returnType) (expressions.h:243-266): takes ownership of the n_args
 * argument trees.  The join filter compiles "substr" (2 or 3 arguments: a string, then INT or
 * LONG start and length in UTF-8 code points; stringfunctions.h:215-318) under the substr
 * policies in force when the join factory is created. */
int32_t omg_expr_func(const char *name, void *const *args, int32_t n_args, const OmgDataType *return_type,
    void **out_expr);
int32_t omg_expr_binary(int32_t op, void *left, void *right, void **out_expr);
/* BinaryExpr with an explicit return type (the reference's BinaryExpr(op, left, right, type)),
 * for arithmetic nodes (ADD .. TRY_DIV: the result is INT, LONG or DOUBLE). */
int32_t omg_expr_binary_typed(int32_t op, void *left, void *right, const OmgDataType *type, void **out_expr);
int32_t omg_expr_unary(int32_t op, void *child, void **out_expr);
/* IfExpr(cond, texp, fexp), SwitchExpr(whens, fexp) (n_whens pairs conds[i] -> results[i]),
 * CoalesceExpr(val1, val2), InExpr(args: the value, then the list), BetweenExpr(val, low, up)
 * (expressions.h:166-230); each takes ownership of its children.  Semantics as the reference's
 * row code generator (codegen/expression_codegen.cpp:352-760): IF / CASE take a branch only on
 * TRUE; IN is TRUE on a match, else NULL when the value or an item is NULL; BETWEEN is NULL when
 * any operand is NULL.  IN and BETWEEN take INT, LONG, DATE32, TIMESTAMP, DOUBLE, VARCHAR, CHAR. */
int32_t omg_expr_if(void *cond, void *then_expr, void *else_expr, void **out_expr);
int32_t omg_expr_switch(void *const *conds, void *const *results, int32_t n_whens, void *else_expr, void **out_expr);
int32_t omg_expr_coalesce(void *value1, void *value2, void **out_expr);
int32_t omg_expr_in(void *const *args, int32_t n_args, void **out_expr);
int32_t omg_expr_between(void *value, void *lower, void *upper, void **out_expr);
int32_t omg_expr_is_null(void *child, void **out_expr);
int32_t omg_expr_free(void *expr);

/* OperatorFactory::CreateOperator (operator/operator_factory.h:18). */
int32_t omg_factory_create_operator(void *factory, void **out_op);
/* Factory destructor (the JNI closeNative on a factory). */
int32_t omg_factory_destroy(void *factory);

/* ---- operators ---------------------------------------------------------------------- */
/* Operator::Init (operator/operator.h:56). */
int32_t omg_op_init(void *op);
/* Operator::AddInput (operator.h:36).  Takes ownership of `batch` as the reference does
 * (group_aggregation.cpp:395-396, lookup_join.cpp:464-466; the builder retains it).
 * `*ret` receives the reference's int32 return value (0). */
int32_t omg_op_add_input(void *op, void *batch, int32_t *ret);
/* Operator::GetOutput (operator.h:38).  `*out_batch` is NULL or a new batch owned by the
 * caller; `*ret` is the reference's return value (agg: 1 if a batch was produced). */
int32_t omg_op_get_output(void *op, void **out_batch, int32_t *ret);
/* Bulk forms with no reference counterpart (a native caller makes the per-batch calls above;
 * these exist so that a caller behind a slow FFI, such as ctypes, pays one crossing for many
 * batches).  omg_op_add_inputs is n calls of Operator::AddInput in order: it stops at the
 * first error, and `*consumed` receives how many batches the operator took (the failing batch
 * counts as taken, as AddInput frees it; later batches stay with the caller).
 * omg_op_get_outputs calls Operator::GetOutput until it yields no batch or `max` batches were
 * returned; `*n` receives the count and `*rows` (may be NULL) their total row count. */
int32_t omg_op_add_inputs(void *op, void *const *batches, int32_t n, int32_t *consumed);
int32_t omg_op_get_outputs(void *op, void **out_batches, int32_t max, int32_t *n, int64_t *rows);
/* Frees n batches (VectorHelper::FreeVecBatch each); NULL entries are skipped. */
int32_t omg_batch_free_many(void *const *batches, int32_t n);
/* Sizing record of a HashAggregation operator (no reference counterpart): [0] rows of the first
 * flush, [1..16] the key sketch of a row sample of that flush (sampled rows, special-key rows,
 * distinct hashes, frequency classes f1, f2, f3, f4-7, f8+, largest count, rows of the 8+
 * class, 6 reserved), [17] the group estimate used for sizing, [18] the partition bits of the
 * partitioned strategy (-1 = global table), [19] the group count so far, [20] the plain
 * (sketch) estimate, [21] 1 if a sizing model made the estimate used, [22] 1 if a shared-memory
 * front table sat before the global one (OMG_AGG_STRATEGY_SMEM).
 * `*written` receives the number of values stored (at most n). */
int32_t omg_op_get_sizing_log(void *op, int64_t *out, int32_t n, int32_t *written);
/* ---- learned sizing model (no reference counterpart) ---------------------------------
 * A small fully connected network (ReLU hidden layers, one output) that maps the features of a
 * sizing record (omg_op_get_sizing_log) to a group-count estimate.  Parameters live in HBM;
 * forward, backward and Adam run as CUDA kernels.  dims = {12, hidden..., 1}.  Host arrays:
 * X is n x dims[0] row-major, T and Y have n entries, parameters are the layers' W (dims[l] x
 * dims[l+1], row-major) and b in layer order. */
int32_t omg_sizer_create(const int32_t *dims, int32_t n_dims, uint64_t seed, void **out_model);
int32_t omg_sizer_destroy(void *model);
int32_t omg_sizer_num_params(void *model, int64_t *n_params);
int32_t omg_sizer_get_params(void *model, float *params, int64_t n_params);
int32_t omg_sizer_set_params(void *model, const float *params, int64_t n_params);
int32_t omg_sizer_predict(void *model, const float *X, int32_t n, float *Y);
/* Gradient of the mean squared error over the batch; *loss receives the loss. */
int32_t omg_sizer_gradients(void *model, const float *X, const float *T, int32_t n, float *grad, float *loss);
/* `epochs` full-batch Adam steps at learning rate lr; *loss receives the loss of the last step. */
int32_t omg_sizer_train(void *model, const float *X, const float *T, int32_t n, int32_t epochs, float lr,
    float *loss);
/* Feature vector (12 floats) of a sizing record of n_log >= 17 values; the training target of a
 * record whose true group count is `groups`; the estimate of a model output y. */
int32_t omg_sizer_features(const int64_t *sizing_log, int32_t n_log, float *features);
int32_t omg_sizer_target(const int64_t *sizing_log, int32_t n_log, int64_t groups, float *target);
int32_t omg_sizer_estimate(const int64_t *sizing_log, int32_t n_log, float y, int64_t *estimate);
/* Attach a model to a HashAggregation factory: operators created afterwards size their table
 * and choose their strategy from the model's estimate instead of the plain sketch estimate
 * (the exact resize path still corrects any misprediction).  NULL detaches.  The model must
 * outlive those operators. */
int32_t omg_hashagg_factory_set_sizer(void *factory, void *model);
/* ---- batched aggregation of many tasks (no reference counterpart) ---------------------
 * The reference runs one HashAggregation operator per task.  These entry points run n tasks of
 * one factory's plan (task i = one VectorBatch, aggregated alone) together: per-task tables in
 * one slab sized by a batched key sketch or by `sizer` (may be NULL), one persistent kernel over
 * all tasks' tiles with an autotuned launch shape, the whole per-run sequence captured once as a
 * CUDA graph and replayed by every omg_agg_batch_run.  A task whose groups outgrow its table is
 * re-run through a regular operator, so results equal n separate operators.  The task batches
 * stay owned by the caller and must outlive the batch object.  Plans with sticky-overflow sums
 * (decimal SUM, generic-policy int64 SUM) are rejected with OMG_ERR_UNSUPPORTED. */
#define OMG_BATCH_DEVICE_OUTPUT 1    /* output batches stay in HBM */
#define OMG_BATCH_NO_GRAPH 2         /* launch the sequence directly instead of a CUDA graph */
#define OMG_BATCH_NO_TUNE 4          /* default launch shape */
#define OMG_BATCH_DEBUG_TINY_TABLES 8 /* tests: 64-slot tables, overflowing tasks re-run by operators */
#define OMG_BATCH_DEBUG_TINY_GROW 16  /* tests: 64-slot tables, overflowing tasks take the grow pass */
int32_t omg_agg_batch_create(void *factory, void *const *task_batches, int32_t n_tasks, void *sizer, int32_t flags,
    void **out_batch);
int32_t omg_agg_batch_run(void *batch, void *stream);
/* Output batches of the last run in task order (caller frees each); call until *n == 0.
 * task_of[i] receives the task of out_batches[i]. */
int32_t omg_agg_batch_outputs(void *batch, void **out_batches, int32_t *task_of, int32_t max, int32_t *n);
/* [0] tasks, [1] input rows, [2] table slots, [3] tasks that outgrew their tables and were
 * re-run exactly, [4] threads per CTA, [5] CTAs per SM, [6] runs, [7] groups, [8] tuning us,
 * [9] preparation us, [10] last run's device time us (grow pass included), [11] 1 if a sizing
 * model sized the tables, [12] 1 if runs replay a graph, [13] of [3], tasks finished by the
 * batched grow pass (tables of twice their rows), [14] of [3], tasks re-run through a regular
 * operator. */
int32_t omg_agg_batch_info(void *batch, int64_t *out, int32_t n, int32_t *written);
/* Per task, a sizing record laid out as omg_op_get_sizing_log's (23 values per task). */
int32_t omg_agg_batch_sizing_logs(void *batch, int64_t *out, int64_t n, int64_t *written);
int32_t omg_agg_batch_destroy(void *batch);
/* ---- partitioned join (no reference counterpart) ---------------------------------------
 * LookupJoin probe strategy for the batches processed afterwards: OMG_JOIN_DIRECT (one table,
 * the default), OMG_JOIN_HASH_PARTITIONED or OMG_JOIN_RANGE_PARTITIONED (both sides split into
 * 2^bits partitions, 1 <= bits <= 12, each with its own small table; the range strategy takes
 * 2^bits - 1 sorted splits).  Partitioning applies to unique builds with 8-byte keys, NULL-free
 * build output columns and the probe key as the only probe output column; other shapes keep
 * the direct probe.  The output row multiset does not depend on the strategy. */
#define OMG_JOIN_DIRECT 0
#define OMG_JOIN_HASH_PARTITIONED 1
#define OMG_JOIN_RANGE_PARTITIONED 2
/* OMG_JOIN_LEARNED: learned splits (omg_join_learn_splits) decide the strategy: a run of equal
 * splits longer than 7.5% of the partitions (a key with about 15% of the probe rows) selects the
 * direct probe, which keeps such hot keys in cache; otherwise the hash-partitioned probe with
 * 2^bits partitions. */
#define OMG_JOIN_LEARNED 3
/* OMG_JOIN_QUANTILE: the same choice from exact sample quantiles (omg_join_quantile_splits): a
 * run of equal splits longer than 15% of the partitions selects the direct probe.  No reference
 * counterpart. */
#define OMG_JOIN_QUANTILE 4
int32_t omg_op_set_join_strategy(void *op, int32_t strategy, int32_t bits, const int64_t *splits, int32_t n_splits);
/* The strategy in effect (OMG_JOIN_LEARNED resolved to the one it chose). */
int32_t omg_op_join_strategy(void *op, int32_t *strategy);
/* Range splits learned from a sample of probe keys: a two-stage model of the keys' CDF (a small
 * network trained on the GPU routes each key to a linear leaf); splits are its 1/2^bits quantile
 * crossings.  Writes 2^bits - 1 sorted splits to `splits`. */
int32_t omg_join_learn_splits(const int64_t *sample, int64_t n, int32_t bits, int32_t epochs, uint64_t seed,
    int64_t *splits);
/* Exact sample quantiles as range splits: split k is the sorted sample's key at rank
 * floor(k * n / 2^bits); writes 2^bits - 1 sorted splits.  No reference counterpart. */
int32_t omg_join_quantile_splits(const int64_t *sample, int64_t n, int32_t bits, int64_t *splits);
/* Order-independent fingerprint of the rows of n batches (host or device, same column
 * layout): out[0] = rows, out[1], out[2] = two 64-bit sums of per-row hashes over all columns
 * (NULLs included).  Equal row multisets give equal fingerprints (no reference counterpart;
 * used to compare large outputs on the device). */
int32_t omg_batches_fingerprint(void *const *batches, int32_t n, uint64_t *out);
/* Operator::GetStatus (operator.h:46-49): OMG_STATUS_*. */
int32_t omg_op_status(void *op);
/* Operator::noMoreInput / setNoMoreInput / needsInput (operator.h:117-130). */
int32_t omg_op_no_more_input(void *op);
int32_t omg_op_set_no_more_input(void *op, int32_t no_more_input);
int32_t omg_op_needs_input(void *op);
/* LookupJoinOperator::IsBlocked (lookup_join.cpp:270-277): 1 while the build is unfinished. */
int32_t omg_op_is_blocked(void *op);
/* Operator::GetHashMapUniqueKeys (operator.h:87). */
int64_t omg_op_hashmap_unique_keys(void *op);
/* Operator::AlignSchema (operator.h:92-95; HashAggregationOperator::AlignSchema,
 * group_aggregation.cpp:1182-1218; JNI alignSchemaNative, jni_operator.cpp:249-260): the batch
 * as one-row partial results of a partial aggregation (every aggregator raw input, partial
 * output), written to `*out`; the input batch is freed whatever the status.  Operators without
 * a partial schema hand the batch back unchanged. */
int32_t omg_op_align_schema(void *op, void *batch, void **out);
/* Operator::Close (operator.h:61) and Operator::DeleteOperator (operator.h:40-44). */
int32_t omg_op_close(void *op);
int32_t omg_op_delete(void *op);

/* ---- GB300-specific operator controls (no reference counterpart) --------------------- */
/* Run the operator's kernels on `stream` (a cudaStream_t; NULL = the operator's own). */
int32_t omg_op_set_stream(void *op, void *stream);
/* 1: GetOutput returns DEVICE vectors (HBM) instead of host vectors. */
int32_t omg_op_set_device_output(void *op, int32_t on);
/* Aggregation: strategy hint and initial global-table capacity (groups); 0 = automatic. */
int32_t omg_op_set_agg_strategy(void *op, int32_t strategy, int64_t capacity_hint);
/* How an aggregation operator estimates its group count when no capacity hint is given
 * (no reference counterpart): OMG_AGG_SIZING_SAMPLE (default) -- the key sketch of a 65,536-row
 * sample, with the factory's sizing model when one is set; OMG_AGG_SIZING_HLL -- a HyperLogLog
 * sketch (2^14 registers) of every row's key, one extra pass over the keys.  Results never
 * depend on it. */
#define OMG_AGG_SIZING_SAMPLE 0
#define OMG_AGG_SIZING_HLL 1
int32_t omg_op_set_agg_sizing(void *op, int32_t mode);
/* Aggregation spill (SpillConfig, core/src/operator/config/operator_config.h:28-100): with
 * enabled != 0 the operator stages its input until GetOutput and, when the estimated group table
 * would exceed device_budget_bytes, hash-partitions the rows into pinned host memory and
 * aggregates one partition at a time.  Call before the first AddInput.  Plans with VARCHAR/CHAR
 * columns or order-dependent sticky-overflow sums return OMG_ERR_UNSUPPORTED. */
int32_t omg_op_set_spill(void *op, int32_t enabled, int64_t device_budget_bytes);
/* Operator::GetSpilledBytes (core/src/operator/operator.h:66): bytes moved to host memory. */
int64_t omg_op_spilled_bytes(void *op);
/* Counters of the last run: [0]=kernel launches, [1]=table resizes, [2]=retried rows,
 * [3]=groups, [4]=ordered-fallback groups, [5]=output rows, [6]=kernel ns, [7]=timed kernel
 * launches; LookupJoin host time: [8]=ns setting up and launching probe calls, [9]=ns waiting
 * for their kernels, [10]=ns carving output batches, [11]=ns freeing probe input batches. */
int32_t omg_op_get_counters(void *op, int64_t *out, int32_t n);

/* ---- allocation-free aggregation (no counterpart in the reference) ----------------------
 * Runs the aggregation compiled by a hash aggregation factory over one batch of
 * device-resident columns without allocating any memory, device or host.  For callers that
 * cannot let this library allocate: a host engine that accounts for every byte of device
 * memory in its own pre-reserved pool, or code running where allocation calls are not allowed.
 * The group table and launch descriptors live in a fixed 64 MiB device array inside the
 * library (held by every GPU that loads it, until the process exits); a call is rejected with
 * OMG_ERR_INVALID_ARG when max_groups and n_rows would not fit in it, or when the input turns
 * out to have more than max_groups groups (num_groups is then left unchanged); a bounded
 * device-side wait that ran out returns OMG_ERR_TIMEOUT (omg_debug_set_wait_budget applies).
 *   d_cols[n_cols], d_nulls[n_cols]: device values / null bitmaps by batch column index
 *     (d_nulls or an entry may be NULL: no nulls); the factory's column indices select from them.
 *   d_out_values[n_out], d_out_nulls[n_out]: the caller's device output columns (group-by
 *     columns, then one per aggregate, in the factory's output order) with room for max_groups
 *     rows; null bitmaps need ((max_groups + 31) / 32) * 4 bytes and are cleared by the call.
 *   *num_groups receives the number of rows written.  The call synchronises `stream`.
 * The first call on a device looks up the device address of the array for that device; make
 * that first call before any stream capture.  Every call shares the array, so calls that overlap
 * on the GPU (e.g. issued concurrently on two streams) race on it and must be serialised by the
 * caller.  Order-dependent sticky overflows (generic-policy int64 SUM, decimal128 SUM) that
 * would need the operator's ordered replay return OMG_ERR_UNSUPPORTED. */
int32_t omg_hashagg_run_noalloc(void *factory, const void *const *d_cols, const uint8_t *const *d_nulls,
    int32_t n_cols, int64_t n_rows, void *const *d_out_values, uint8_t *const *d_out_nulls, int32_t n_out,
    int64_t max_groups, int64_t *num_groups, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* OMNIOP_GB300_H */
