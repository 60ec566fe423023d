// HashAggregationOperatorFactory / HashAggregationOperator (see omniop/hash_aggregation.h).
//
// Plan compilation follows the reference's aggregator selection
// (operator/aggregation/aggregation.cpp:20-88, aggregator/aggregator_factory.cpp:78-125):
//  Spark policy (default):  SUM int -> wrapping int64 (sum_flatim_aggregator.h:33),
//                           SUM decimal -> exact with sticky overflow (sum_spark_decimal_aggregator.h),
//                           AVG -> double sum / count (average_flatim_aggregator.h:225-290);
//  generic policy:          SUM int64 -> exact with sticky overflow (sum_aggregator.h:43-49).
// COUNT, MIN and MAX are policy independent (count_*_aggregator.h, min/max_aggregator.h).
#include "omniop/hash_aggregation.h"

#include <algorithm>
#include <cmath>
#include <cfloat>
#include <climits>
#include <cstring>
#include <map>

#include "host/gpu_runtime.h"
#include "host/sizer.h"
#include "kernels/launch.h"

namespace omniruntime {
namespace op {

using omg::AccSpec;
using omg::CudaCheck;
using omg::DevArray;
using omg::OutSpec;
using exception::OmniException;
using namespace type;

namespace {

bool IsIntegerLike(DataTypeId id)
{
    switch (id) {
        case OMNI_BYTE:
        case OMNI_BOOLEAN:
        case OMNI_SHORT:
        case OMNI_INT:
        case OMNI_LONG:
        case OMNI_DATE32:
        case OMNI_DATE64:
        case OMNI_TIMESTAMP:
        case OMNI_DECIMAL64:
            return true;
        default:
            return false;
    }
}

int64_t IntMaxForWidth(int w)
{
    switch (w) {
        case 1:
            return INT8_MAX;
        case 2:
            return INT16_MAX;
        case 4:
            return INT32_MAX;
        default:
            return INT64_MAX;
    }
}
int64_t IntMinForWidth(int w)
{
    switch (w) {
        case 1:
            return INT8_MIN;
        case 2:
            return INT16_MIN;
        case 4:
            return INT32_MIN;
        default:
            return INT64_MIN;
    }
}

int64_t OrderedBits(double x)
{
    int64_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

bool IsVarlen(DataTypeId id) { return id == OMNI_VARCHAR || id == OMNI_CHAR; }

// Bytes a VARCHAR/CHAR value counts for in the output batch size rule: the declared width, or
// 200 when none is declared (operator_util.h:72-82).
int VarlenRowBytes(const DataTypePtr &t)
{
    const int32_t w = t->GetWidth();
    const int32_t unset = t->GetId() == OMNI_CHAR ? 65536 : INT_MAX;
    return w > 0 && w < unset ? w : 200;
}

uint64_t NextPow2(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) {
        p <<= 1;
    }
    return p;
}

constexpr uint64_t kDefaultCapacity = uint64_t(1) << 16;
constexpr int kGlobalMaxProbe = 96;
constexpr size_t kSmemBudget = 96 * 1024;            // shared bytes per CTA for pre-aggregation

}  // namespace

// ------------------------------------------------------------------------------ factory
HashAggregationOperatorFactory::HashAggregationOperatorFactory(std::vector<uint32_t> &groupByCol,
    const DataTypes &groupInputTypes, std::vector<std::vector<uint32_t>> &aggsCols,
    std::vector<DataTypes> &aggInputTypes, std::vector<DataTypes> &aggOutputTypes,
    std::vector<uint32_t> &aggFuncTypes, std::vector<uint32_t> &maskColsVector, std::vector<bool> inputRaws,
    std::vector<bool> outputPartials, bool overflowAsNull)
    : groupByCols_(groupByCol), groupTypes_(groupInputTypes), aggCols_(aggsCols), aggInputTypes_(aggInputTypes),
      aggOutputTypes_(aggOutputTypes), aggFuncTypes_(aggFuncTypes), maskCols_(maskColsVector),
      inputRaws_(std::move(inputRaws)), outputPartials_(std::move(outputPartials)), overflowAsNull_(overflowAsNull),
      policy_(GetSupportContainerVecRule())
{}

OmniStatus HashAggregationOperatorFactory::Init()
{
    if (inited_) {
        return OMNI_STATUS_NORMAL;
    }
    const size_t nAgg = aggFuncTypes_.size();
    if (groupByCols_.size() != static_cast<size_t>(groupTypes_.GetSize()) || groupByCols_.empty()) {
        throw OmniException("INVALID_ARGUMENT", "group-by columns and types disagree", -1);
    }
    if (aggCols_.size() != nAgg || aggInputTypes_.size() != nAgg || aggOutputTypes_.size() != nAgg) {
        throw OmniException("INVALID_ARGUMENT", "aggregator columns/types/functions disagree", -1);
    }
    // Mask columns (aggregation.cpp:12-18, MaskColAggregator): aggregator a sees only the rows
    // whose BOOLEAN column maskCols_[a] is TRUE (a NULL mask counts as FALSE); UINT32_MAX (the
    // reference's static_cast<uint32_t>(-1)) means no mask.  Every row still creates its group.
    if (!maskCols_.empty() && maskCols_.size() != nAgg) {
        throw OmniException("INVALID_ARGUMENT", "one mask column entry per aggregator is required", -1);
    }
    auto maskOf = [&](size_t a) {
        return a < maskCols_.size() && maskCols_[a] != UINT32_MAX ? static_cast<int32_t>(maskCols_[a]) : -1;
    };

    AggPlan &p = plan_;
    p = AggPlan();
    p.overflowAsNull = overflowAsNull_;
    // (batch column, mask column or -1) -> kernel input.  A masked input reads the column's values
    // with the rows its mask drops turned into NULLs (BatchTable builds that bitmap), so every
    // accumulator, strategy and merge handles masks the way it handles NULL values.
    std::map<std::pair<uint32_t, int32_t>, int32_t> inputOf;
    auto inputFor = [&](uint32_t col, int width, int32_t mask = -1) {
        auto it = inputOf.find(std::make_pair(col, mask));
        if (it != inputOf.end()) {
            p.inputWidths[it->second] = std::max(p.inputWidths[it->second], width);
            return it->second;
        }
        const int32_t idx = static_cast<int32_t>(p.inputCols.size());
        if (idx >= omg::kMaxInputs) {
            throw OmniException("UNSUPPORTED_ERROR", "too many distinct input columns", -2);
        }
        p.inputCols.push_back(static_cast<int32_t>(col));
        p.inputWidths.push_back(width);
        p.inputMasks.push_back(mask);
        inputOf[std::make_pair(col, mask)] = idx;
        return idx;
    };

    // ---- key
    const int nKey = static_cast<int>(groupByCols_.size());
    if (nKey > omg::kMaxKeyCols) {
        throw OmniException("UNSUPPORTED_ERROR", "at most 4 group-by columns are supported", -2);
    }
    std::memset(&p.key, 0, sizeof(p.key));
    p.key.nCols = nKey;
    int rowBytes = 0;
    for (int i = 0; i < nKey; ++i) {
        const auto &t = groupTypes_.GetType(i);
        // A VARCHAR/CHAR key is aggregated as the int32 id of its string in the operator's
        // string dictionary (the reference serialises the bytes into the key instead,
        // vector_marshaller.cpp:155-232); the strings come back at output time.
        const bool varlen = IsVarlen(t->GetId());
        const int w = varlen ? 4 : t->ByteWidth();
        if (w == 0 || (w > 8 && w != 16)) {
            throw OmniException("UNSUPPORTED_ERROR", "unsupported group-by type " + std::to_string(t->GetId()), -2);
        }
        const int32_t input = inputFor(groupByCols_[i], w);
        if (varlen && std::find(p.dictInputs.begin(), p.dictInputs.end(), input) == p.dictInputs.end()) {
            p.dictInputs.push_back(input);
        }
        p.key.cols[i].input = static_cast<int16_t>(input);
        p.key.cols[i].width = static_cast<int16_t>(w);
        p.outTypes.push_back(t);
        rowBytes += varlen ? VarlenRowBytes(t) : w;
    }
    if (nKey == 1 && p.key.cols[0].width <= 8) {
        p.key.kind = omg::KEY_SINGLE;
        p.key.words = 1;
        p.keyWords = 1;
    } else {
        // Pack widest first at natural alignment so no value straddles a word.
        std::vector<int> order(nKey);
        for (int i = 0; i < nKey; ++i) {
            order[i] = i;
        }
        std::stable_sort(order.begin(), order.end(),
            [&](int a, int b) { return p.key.cols[a].width > p.key.cols[b].width; });
        int off = 0;
        for (int i : order) {
            p.key.cols[i].byteOffset = static_cast<int16_t>(off);
            off += p.key.cols[i].width;
        }
        p.key.maskByte = off;
        const int bytes = off + 1;
        if (bytes > 24) {
            throw OmniException("UNSUPPORTED_ERROR", "packed group-by key wider than 23 bytes", -2);
        }
        p.key.kind = omg::KEY_PACKED;
        p.key.words = (bytes + 7) / 8;
        p.keyWords = 1 + p.key.words;  // tag + key words
    }

    // ---- accumulators
    std::map<std::pair<int, int>, int> accOf;  // (kind, input) -> acc index
    int word = 0;
    auto accFor = [&](int kind, int input, int inKind, int inWidth, int64_t init) {
        auto key = std::make_pair(kind, input);
        auto it = accOf.find(key);
        if (it != accOf.end()) {
            return it->second;
        }
        if (static_cast<int>(p.accs.size()) >= omg::kMaxAccs) {
            throw OmniException("UNSUPPORTED_ERROR", "too many aggregate states", -2);
        }
        AccSpec a{};
        a.kind = static_cast<int16_t>(kind);
        a.input = static_cast<int16_t>(input);
        a.inKind = static_cast<int16_t>(inKind);
        a.inWidth = static_cast<int16_t>(inWidth);
        if ((kind == omg::ACC_XMIN || kind == omg::ACC_XMAX) && ((p.keyWords + word) & 1) != 0) {
            ++word;  // 16-byte states sit on a 16-byte boundary of the (even-sized) slot
        }
        a.word = word;
        a.init = init;
        word += omg::AccWords(kind);
        p.accs.push_back(a);
        const int idx = static_cast<int>(p.accs.size()) - 1;
        accOf[key] = idx;
        return idx;
    };
    accFor(omg::ACC_COUNT_ALL, -1, omg::IN_NONE, 0, 0);  // always accs[0]

    // Output key columns.
    for (int i = 0; i < nKey; ++i) {
        OutSpec o{};
        o.kind = omg::OUT_KEY;
        o.src = static_cast<int16_t>(i);
        o.countAcc = -1;
        o.outWidth = p.key.cols[i].width;
        o.outType = static_cast<int16_t>(groupTypes_.GetType(i)->GetId());
        p.outs.push_back(o);
    }
    int exactIndex = 0;
    const bool spark = policy_ == SupportContainerVecRule::NOT_SUPPORT;
    // Two-stage aggregation (group_aggregation.cpp:1182-1218): a partial stage (outputPartial)
    // emits per-group intermediate values, a final stage (inputRaw = false) merges them.  SUM,
    // MIN and MAX partials are their plain results; COUNT partials are counts the final stage
    // sums (never NULL); an AVG partial is two columns, the double sum (0 for a group without
    // values) and the count, and the final AVG is their summed sum over their summed count
    // (average_flatim_aggregator.h:81-175,225-290, count_column_aggregator.cpp:54-160).
    auto pushOut = [&](OutSpec o, const DataTypePtr &t) {
        o.outType = static_cast<int16_t>(t->GetId());
        o.outWidth = static_cast<int16_t>(t->ByteWidth());
        p.outs.push_back(o);
        p.outTypes.push_back(t);
        rowBytes += o.outWidth;
    };
    std::vector<size_t> containerAt;  // outs that start a two-field container output
    // The (double sum, count) pair of a partial AVG: two flat outputs of the given types, or
    // (avgContainer) the fields of one container output.
    auto pushAvgPair = [&](const OutSpec &s1, const OutSpec &s2, const DataTypes &outTypes, bool avgContainer) {
        if (avgContainer) {
            containerAt.push_back(p.outs.size());
            pushOut(s1, DoubleType());
            pushOut(s2, LongType());
        } else {
            pushOut(s1, outTypes.GetType(0));
            pushOut(s2, outTypes.GetType(1));
        }
    };
    for (size_t a = 0; a < nAgg; ++a) {
        const uint32_t fn = aggFuncTypes_[a];
        const bool raw = a < inputRaws_.size() ? static_cast<bool>(inputRaws_[a]) : true;
        const bool partial = a < outputPartials_.size() ? static_cast<bool>(outputPartials_[a]) : false;
        const auto &outTypes = aggOutputTypes_[a];
        const bool avgPair = fn == OMNI_AGGREGATION_TYPE_AVG && partial;
        const DataTypeId in0 = aggInputTypes_[a].GetSize() > 0 ? aggInputTypes_[a].GetType(0)->GetId() : OMNI_NONE;
        const bool decSum = fn == OMNI_AGGREGATION_TYPE_SUM && (in0 == OMNI_DECIMAL64 || in0 == OMNI_DECIMAL128);
        const bool decPair = decSum && partial;
        // A partial AVG under the container-vector policy (average_aggregator.cpp:13-38): one
        // CONTAINER output of (double sum, long count) fields in place of the two flat columns.
        const bool avgContainer = avgPair && outTypes.GetSize() == 1 && outTypes.GetType(0)->GetId() == OMNI_CONTAINER;
        for (int32_t t = 0; t < outTypes.GetSize() && !avgContainer; ++t) {
            if (outTypes.GetType(t)->GetId() == OMNI_CONTAINER) {
                throw OmniException("INVALID_ARGUMENT", "only a partial AVG emits a container column", -1);
            }
        }
        for (int32_t t = 0; t < aggInputTypes_[a].GetSize(); ++t) {
            if (aggInputTypes_[a].GetType(t)->GetId() == OMNI_CONTAINER &&
                !(fn == OMNI_AGGREGATION_TYPE_AVG && !raw && aggInputTypes_[a].GetSize() == 1)) {
                throw OmniException("INVALID_ARGUMENT", "only a merging AVG reads a container column", -1);
            }
        }
        if (!avgContainer && outTypes.GetSize() != (avgPair || decPair ? 2 : 1)) {
            throw OmniException("INVALID_ARGUMENT",
                avgPair ? "a partial AVG has two output types (double sum, long count)"
                        : (decPair ? "a partial decimal SUM has two output types (decimal sum, boolean isEmpty)"
                                   : "this aggregator has one output type"), -1);
        }
        const DataTypePtr &outT = outTypes.GetType(0);
        OutSpec o{};
        o.outType = static_cast<int16_t>(outT->GetId());
        o.outWidth = static_cast<int16_t>(outT->ByteWidth());
        o.countAcc = -1;
        const int32_t mask = maskOf(a);
        if (!raw && (fn == OMNI_AGGREGATION_TYPE_COUNT_ALL || fn == OMNI_AGGREGATION_TYPE_COUNT_COLUMN)) {
            // final COUNT / COUNT(*): the sum of the partial counts
            if (aggCols_[a].size() != 1 || aggInputTypes_[a].GetSize() != 1 ||
                !IsIntegerLike(aggInputTypes_[a].GetType(0)->GetId())) {
                throw OmniException("INVALID_ARGUMENT", "a final COUNT reads one integer column of partial counts", -1);
            }
            const int in = inputFor(aggCols_[a][0], aggInputTypes_[a].GetType(0)->ByteWidth(), mask);
            accFor(omg::ACC_NULLS, in, omg::IN_NONE, 0, 0);
            o.kind = omg::OUT_COUNT_MERGE;
            o.src = static_cast<int16_t>(
                accFor(omg::ACC_ISUM, in, omg::IN_INT, aggInputTypes_[a].GetType(0)->ByteWidth(), 0));
            pushOut(o, outT);
            continue;
        }
        if (fn == OMNI_AGGREGATION_TYPE_COUNT_ALL) {
            o.kind = omg::OUT_COUNT;
            o.src = 0;
            if (mask >= 0) {
                // COUNT(*) of the rows the mask keeps: COUNT_ALL minus the NULLs of the mask
                // column read through its own mask (its NULL and FALSE rows).
                o.countAcc = static_cast<int16_t>(
                    accFor(omg::ACC_NULLS, inputFor(static_cast<uint32_t>(mask), 1, mask), omg::IN_NONE, 0, 0));
                o.boundKind = 2;  // marks a masked COUNT(*) (AlignSchema emits 1 for it)
            }
            p.outs.push_back(o);
            p.outTypes.push_back(outT);
            rowBytes += o.outWidth;
            continue;
        }
        if (fn == OMNI_AGGREGATION_TYPE_AVG && (in0 == OMNI_DECIMAL64 || in0 == OMNI_DECIMAL128)) {
            // Spark decimal AVG (AverageSparkDecimalAggregator, average_spark_decimal_aggregator.h):
            // a checked sum with sticky overflow -- int64 for a decimal64 input and output,
            // within +-(10^38 - 1) otherwise -- and the non-NULL count.  A partial emits (sum
            // rescaled to the output scale, count): 0 and 0 for a group without values, the sum
            // NULL (or an error) on overflow; a merging stage adds the partial sums (checked) and
            // counts, skipping rows whose partial sum is NULL; the final value is CalcAvg (:477).
            if (!spark) {
                throw OmniException("UNSUPPORTED_ERROR", "decimal AVG under the container-vector policy is not supported",
                    -2);
            }
            const DataTypePtr &inT = aggInputTypes_[a].GetType(0);
            const int inW = inT->ByteWidth();
            const int inKind = in0 == OMNI_DECIMAL128 ? omg::IN_DEC128 : omg::IN_INT;
            const int accKind = in0 == OMNI_DECIMAL128 ? omg::ACC_WSUM3 : omg::ACC_WSUM2;
            // The sum's bound: int64 when both the input and the intermediate are decimal64.
            const DataTypeId midId = partial ? outTypes.GetType(0)->GetId() : outT->GetId();
            const int16_t bound = (in0 == OMNI_DECIMAL64 && midId == OMNI_DECIMAL64) ? 0 : 1;
            int sumAcc;
            int cntAcc;
            bool summed;
            if (raw) {
                if (aggCols_[a].size() != 1 || aggInputTypes_[a].GetSize() != 1) {
                    throw OmniException("INVALID_ARGUMENT", "a decimal AVG reads one decimal column", -1);
                }
                const int input = inputFor(aggCols_[a][0], inW, mask);
                cntAcc = accFor(omg::ACC_NULLS, input, omg::IN_NONE, 0, 0);
                sumAcc = accFor(accKind, input, inKind, inW, 0);
                summed = false;
            } else {
                if (aggCols_[a].size() != 2 || aggInputTypes_[a].GetSize() != 2 ||
                    !IsIntegerLike(aggInputTypes_[a].GetType(1)->GetId())) {
                    throw OmniException("INVALID_ARGUMENT", "a merging decimal AVG reads (decimal sum, long count) partial columns",
                        -1);
                }
                if (mask >= 0) {
                    throw OmniException("UNSUPPORTED_ERROR", "a mask column on a merging decimal AVG is not supported", -2);
                }
                const int sums = inputFor(aggCols_[a][0], inW);
                const int cntW = aggInputTypes_[a].GetType(1)->ByteWidth();
                const int counts = inputFor(aggCols_[a][1], cntW, omg::NullsOfMask(static_cast<int32_t>(aggCols_[a][0])));
                accFor(omg::ACC_NULLS, sums, omg::IN_NONE, 0, 0);
                sumAcc = accFor(accKind, sums, inKind, inW, 0);
                cntAcc = accFor(omg::ACC_ISUM, counts, omg::IN_INT, cntW, 0);
                summed = true;
            }
            OutSpec s1{};
            s1.src = static_cast<int16_t>(sumAcc);
            s1.countAcc = static_cast<int16_t>(cntAcc);
            s1.countSummed = summed ? 1 : 0;
            s1.boundKind = bound;
            s1.pad = static_cast<int16_t>(exactIndex++);
            if (partial) {
                // (sum, count): the sum rescaled to the partial's output scale
                // (ExtractValues, :276-295); a partial of p digits is declared (p + 10, s).
                const DataTypePtr &sumT = outTypes.GetType(0);
                const int diff = sumT->GetScale() - inT->GetScale();
                if (diff < 0 || diff > 38) {
                    throw OmniException("UNSUPPORTED_ERROR", "decimal AVG partial scale below input scale", -2);
                }
                s1.kind = omg::OUT_SUM_EXACT;
                s1.boundKind = sumT->GetId() == OMNI_DECIMAL128 ? bound : 0;
                s1.rescalePow = static_cast<int16_t>(diff);
                s1.partial = 2;
                pushOut(s1, sumT);
                OutSpec s2{};
                s2.kind = summed ? omg::OUT_COUNT_MERGE : omg::OUT_COUNT;
                s2.src = summed ? static_cast<int16_t>(cntAcc) : 0;
                s2.countAcc = summed ? -1 : static_cast<int16_t>(cntAcc);
                pushOut(s2, outTypes.GetType(1));
                continue;
            }
            if (outT->GetId() != OMNI_DECIMAL64 && outT->GetId() != OMNI_DECIMAL128) {
                throw OmniException("UNSUPPORTED_ERROR", "decimal AVG needs a decimal output type", -2);
            }
            s1.kind = omg::OUT_AVG_DEC;
            // A single-stage AVG sums at precision p + 10 (CalcAvg, :485-488); a final stage sums
            // the partial sums at their declared precision.
            s1.sumPrec = static_cast<int16_t>(raw ? std::min(inT->GetPrecision() + 10, 38) : inT->GetPrecision());
            s1.sumScale = static_cast<int16_t>(inT->GetScale());
            s1.rescalePow = static_cast<int16_t>(outT->GetScale());
            pushOut(s1, outT);
            continue;
        }
        if (fn == OMNI_AGGREGATION_TYPE_AVG && !raw) {
            // final AVG over (double sum, long count) partial columns, or over the fields of one
            // CONTAINER column (average_aggregator.cpp:230-300)
            const bool fromContainer = aggCols_[a].size() == 1 && aggInputTypes_[a].GetSize() == 1 &&
                aggInputTypes_[a].GetType(0)->GetId() == OMNI_CONTAINER;
            if (!fromContainer &&
                (aggCols_[a].size() != 2 || aggInputTypes_[a].GetSize() != 2 ||
                    aggInputTypes_[a].GetType(0)->GetId() != OMNI_DOUBLE ||
                    !IsIntegerLike(aggInputTypes_[a].GetType(1)->GetId()))) {
                throw OmniException("INVALID_ARGUMENT",
                    "a final AVG reads (double sum, long count) partial columns or one container column", -1);
            }
            const int cntW = fromContainer ? 8 : aggInputTypes_[a].GetType(1)->ByteWidth();
            const int inSum = fromContainer ? inputFor(static_cast<uint32_t>(omg::FieldRef(aggCols_[a][0], 0)), 8, mask)
                                            : inputFor(aggCols_[a][0], 8, mask);
            const int inCnt = fromContainer ? inputFor(static_cast<uint32_t>(omg::FieldRef(aggCols_[a][0], 1)), 8, mask)
                                            : inputFor(aggCols_[a][1], cntW, mask);
            accFor(omg::ACC_NULLS, inSum, omg::IN_NONE, 0, 0);
            accFor(omg::ACC_NULLS, inCnt, omg::IN_NONE, 0, 0);
            const int sumAcc = accFor(omg::ACC_DSUM, inSum, omg::IN_DOUBLE, 8, 0);
            const int cntAcc = accFor(omg::ACC_ISUM, inCnt, omg::IN_INT, cntW, 0);
            if (partial) {  // an intermediate merge: still (sum, count)
                OutSpec s1{};
                s1.kind = omg::OUT_AVG_PARTIAL_SUM;
                s1.src = static_cast<int16_t>(sumAcc);
                s1.countAcc = static_cast<int16_t>(cntAcc);
                s1.boundKind = 1;  // countAcc holds a summed count
                OutSpec s2{};
                s2.kind = omg::OUT_COUNT_MERGE;
                s2.src = static_cast<int16_t>(cntAcc);
                s2.countAcc = -1;
                pushAvgPair(s1, s2, outTypes, avgContainer);
            } else {
                o.kind = omg::OUT_AVG_MERGE;
                o.src = static_cast<int16_t>(sumAcc);
                o.countAcc = static_cast<int16_t>(cntAcc);
                pushOut(o, outT);
            }
            continue;
        }
        if (decSum && (!raw || partial)) {
            // Spark decimal SUM across stages (sum_spark_decimal_aggregator.h:74-412): a partial
            // emits (sum, isEmpty) -- the sum NULL when it overflowed, 0 for an empty group; a
            // merging stage skips rows whose isEmpty is TRUE, turns a NULL partial sum into a
            // sticky overflow and adds the other partial sums with the same checked, sticky
            // addition (AddDecimalUseRowIndex, :14-66), which the exact sum plus the ordered
            // replay reproduce.
            if (!spark) {
                throw OmniException("UNSUPPORTED_ERROR",
                    "two-stage decimal SUM under the container-vector policy is not supported", -2);
            }
            const DataTypePtr &inT = aggInputTypes_[a].GetType(0);
            const int inW = inT->ByteWidth();
            const int inKind = in0 == OMNI_DECIMAL128 ? omg::IN_DEC128 : omg::IN_INT;
            const int accKind = in0 == OMNI_DECIMAL128 ? omg::ACC_WSUM3 : omg::ACC_WSUM2;
            const int diff = outT->GetScale() - inT->GetScale();
            if (diff < 0 || diff > 38) {
                throw OmniException("UNSUPPORTED_ERROR", "decimal SUM output scale below input scale", -2);
            }
            OutSpec s1{};
            s1.kind = omg::OUT_SUM_EXACT;
            s1.boundKind = outT->GetId() == OMNI_DECIMAL128 ? 1 : 0;
            s1.rescalePow = static_cast<int16_t>(diff);
            s1.pad = static_cast<int16_t>(exactIndex++);
            s1.partial = partial ? 1 : 0;
            if (raw) {
                if (aggCols_[a].size() != 1 || aggInputTypes_[a].GetSize() != 1) {
                    throw OmniException("INVALID_ARGUMENT", "a partial decimal SUM reads one decimal column", -1);
                }
                const int input = inputFor(aggCols_[a][0], inW, mask);
                s1.countAcc = static_cast<int16_t>(accFor(omg::ACC_NULLS, input, omg::IN_NONE, 0, 0));
                s1.src = static_cast<int16_t>(accFor(accKind, input, inKind, inW, 0));
            } else {
                if (aggCols_[a].size() != 2 || aggInputTypes_[a].GetSize() != 2 ||
                    aggInputTypes_[a].GetType(1)->GetId() != OMNI_BOOLEAN) {
                    throw OmniException("INVALID_ARGUMENT",
                        "a merging decimal SUM reads (decimal sum, boolean isEmpty) partial columns", -1);
                }
                if (mask >= 0) {
                    throw OmniException("UNSUPPORTED_ERROR", "a mask column on a merging decimal SUM is not supported",
                        -2);
                }
                const int sums = inputFor(aggCols_[a][0], inW);
                const int kept = inputFor(aggCols_[a][0], inW, omg::InvertedMask(static_cast<int32_t>(aggCols_[a][1])));
                s1.flagAcc = static_cast<int16_t>(accFor(omg::ACC_NULLS, sums, omg::IN_NONE, 0, 0));
                s1.countAcc = static_cast<int16_t>(accFor(omg::ACC_NULLS, kept, omg::IN_NONE, 0, 0));
                s1.src = static_cast<int16_t>(accFor(accKind, kept, inKind, inW, 0));
            }
            pushOut(s1, outT);
            if (partial) {
                OutSpec s2{};
                s2.kind = omg::OUT_IS_EMPTY;
                s2.countAcc = s1.countAcc;
                s2.flagAcc = s1.flagAcc;
                pushOut(s2, outTypes.GetType(1));
            }
            continue;
        }
        if (aggCols_[a].size() != 1 || aggInputTypes_[a].GetSize() != 1) {
            throw OmniException("UNSUPPORTED_ERROR", "aggregator must read exactly one column", -2);
        }
        const DataTypePtr &inT = aggInputTypes_[a].GetType(0);
        const DataTypeId inId = inT->GetId();
        const int inW = inT->ByteWidth();
        const int input = inputFor(aggCols_[a][0], inW, mask);
        const int nulls = accFor(omg::ACC_NULLS, input, omg::IN_NONE, 0, 0);
        o.countAcc = static_cast<int16_t>(nulls);
        const bool isInt = IsIntegerLike(inId);
        const bool isDouble = inId == OMNI_DOUBLE || inId == OMNI_FLOAT;
        const int inKind = inId == OMNI_DOUBLE ? omg::IN_DOUBLE
                                               : (inId == OMNI_FLOAT ? omg::IN_FLOAT
                                                                     : (inId == OMNI_DECIMAL128 ? omg::IN_DEC128 : omg::IN_INT));
        switch (fn) {
            case OMNI_AGGREGATION_TYPE_COUNT_COLUMN:
                o.kind = omg::OUT_COUNT;
                o.src = 0;
                break;
            case OMNI_AGGREGATION_TYPE_SUM: {
                // Under the container-vector policy a two-stage int64 SUM is the same sticky SUM at
                // every stage: a partial emits the sum (NULL when it overflowed or had no values) and
                // a merging stage sums those, skipping NULL rows (sum_aggregator.cpp:11-57,168-190).
                if (isDouble) {
                    o.kind = omg::OUT_SUM_DOUBLE;
                    o.src = static_cast<int16_t>(accFor(omg::ACC_DSUM, input, inKind, inW, 0));
                } else if (inId == OMNI_DECIMAL64 || inId == OMNI_DECIMAL128) {
                    o.kind = omg::OUT_SUM_EXACT;
                    const int kind = inId == OMNI_DECIMAL128 ? omg::ACC_WSUM3 : omg::ACC_WSUM2;
                    o.src = static_cast<int16_t>(accFor(kind, input, inKind, inW, 0));
                    o.boundKind = outT->GetId() == OMNI_DECIMAL128 ? 1 : 0;
                    const int diff = outT->GetScale() - inT->GetScale();
                    if (diff < 0 || diff > 38) {
                        throw OmniException("UNSUPPORTED_ERROR", "decimal SUM output scale below input scale", -2);
                    }
                    o.rescalePow = static_cast<int16_t>(diff);
                    o.pad = static_cast<int16_t>(exactIndex++);
                } else if (isInt) {
                    // SumOp checks overflow only for int64 inputs (sum_aggregator.h:36-60), so
                    // narrower inputs wrap under either policy.
                    if (spark || inW != 8) {
                        o.kind = omg::OUT_SUM_WRAP;
                        o.src = static_cast<int16_t>(accFor(omg::ACC_ISUM, input, inKind, inW, 0));
                    } else {
                        o.kind = omg::OUT_SUM_EXACT;
                        o.src = static_cast<int16_t>(accFor(omg::ACC_WSUM2, input, inKind, inW, 0));
                        o.boundKind = 0;
                        o.pad = static_cast<int16_t>(exactIndex++);
                    }
                } else {
                    throw OmniException("UNSUPPORTED_ERROR", "unsupported SUM input type " + std::to_string(inId), -2);
                }
                break;
            }
            case OMNI_AGGREGATION_TYPE_AVG: {
                if (!isInt && !isDouble) {
                    throw OmniException("UNSUPPORTED_ERROR", "unsupported AVG input type " + std::to_string(inId), -2);
                }
                o.src = static_cast<int16_t>(accFor(omg::ACC_DSUM, input, inKind, inW, 0));
                if (partial) {  // (double sum, long count); 0 and 0 for a group without values
                    OutSpec s1 = o;
                    s1.kind = omg::OUT_AVG_PARTIAL_SUM;
                    s1.countAcc = static_cast<int16_t>(nulls);
                    s1.boundKind = 0;  // countAcc holds the NULL count
                    OutSpec s2{};
                    s2.kind = omg::OUT_COUNT;
                    s2.src = 0;
                    s2.countAcc = static_cast<int16_t>(nulls);
                    pushAvgPair(s1, s2, outTypes, avgContainer);
                    continue;
                }
                o.kind = omg::OUT_AVG;
                break;
            }
            case OMNI_AGGREGATION_TYPE_MIN:
            case OMNI_AGGREGATION_TYPE_MAX: {
                const bool isMin = fn == OMNI_AGGREGATION_TYPE_MIN;
                if (isInt) {
                    const int outW = o.outWidth;
                    o.kind = isMin ? omg::OUT_MIN_INT : omg::OUT_MAX_INT;
                    o.src = static_cast<int16_t>(accFor(isMin ? omg::ACC_IMIN : omg::ACC_IMAX, input, inKind, inW,
                        isMin ? IntMaxForWidth(outW) : IntMinForWidth(outW)));
                } else if (isDouble) {
                    const double lim = inId == OMNI_FLOAT ? static_cast<double>(FLT_MAX) : DBL_MAX;
                    o.kind = isMin ? omg::OUT_MIN_DOUBLE : omg::OUT_MAX_DOUBLE;
                    o.src = static_cast<int16_t>(accFor(isMin ? omg::ACC_DMIN : omg::ACC_DMAX, input, inKind, inW,
                        OrderedBits(isMin ? lim : -lim)));
                } else if (inId == OMNI_DECIMAL128 && outT->GetId() == OMNI_DECIMAL128) {
                    // Decimal128 MIN/MAX (min_aggregator.h, MinAggregator<OMNI_DECIMAL128,
                    // OMNI_DECIMAL128>): a 16-byte state updated by a 128-bit CAS loop.
                    o.kind = omg::OUT_MINMAX_DEC128;
                    o.src = static_cast<int16_t>(
                        accFor(isMin ? omg::ACC_XMIN : omg::ACC_XMAX, input, omg::IN_DEC128, 16, 0));
                } else if (IsVarlen(inId)) {
                    // MIN/MAX of VARCHAR (min_aggregator.cpp / max_aggregator.cpp over string_view):
                    // the input is read as its string dictionary ids and the state keeps the id of
                    // the least / greatest string, compared byte-wise on the device.
                    p.inputWidths[input] = std::max(p.inputWidths[input], 4);
                    if (std::find(p.dictInputs.begin(), p.dictInputs.end(), input) == p.dictInputs.end()) {
                        p.dictInputs.push_back(input);
                    }
                    o.kind = omg::OUT_STR_ID;
                    o.src = static_cast<int16_t>(
                        accFor(isMin ? omg::ACC_SMIN : omg::ACC_SMAX, input, omg::IN_INT, 4, -1));
                    o.outWidth = 4;
                    rowBytes += VarlenRowBytes(outT) - o.outWidth;
                } else {
                    throw OmniException("UNSUPPORTED_ERROR", "unsupported MIN/MAX input type " + std::to_string(inId), -2);
                }
                break;
            }
            default:
                throw OmniException("UNSUPPORTED_ERROR", "No such agg func type " + std::to_string(fn), -2);
        }
        p.outs.push_back(o);
        p.outTypes.push_back(outT);
        rowBytes += o.outWidth;
    }
    if (p.outs.size() > static_cast<size_t>(omg::kMaxOutCols)) {
        throw OmniException("UNSUPPORTED_ERROR", "too many output columns", -2);
    }
    if (exactIndex > 8) {
        throw OmniException("UNSUPPORTED_ERROR", "at most 8 exact SUM columns", -2);
    }
    p.orderDependent = exactIndex > 0;
    // Register cache: the first kRegInputs distinct narrow (<= 8 byte) inputs the accumulators
    // read are loaded once per row, up front.
    for (auto &a : p.accs) {
        a.reg = -1;
        if (a.input < 0 || a.kind == omg::ACC_NULLS || a.inWidth <= 0 || a.inWidth > 8 || a.kind == omg::ACC_WSUM3) {
            continue;
        }
        for (size_t r = 0; r < p.regInput.size(); ++r) {
            if (p.regInput[r] == a.input) {
                a.reg = static_cast<int32_t>(r);
            }
        }
        if (a.reg < 0 && p.regInput.size() < static_cast<size_t>(omg::kRegInputs)) {
            a.reg = static_cast<int32_t>(p.regInput.size());
            p.regInput.push_back(a.input);
            p.regWidth.push_back(a.inWidth);
        }
    }
    // NULLS accumulators of an input share its register slot even though they carry no width.
    for (auto &a : p.accs) {
        if (a.kind == omg::ACC_NULLS) {
            for (size_t r = 0; r < p.regInput.size(); ++r) {
                if (p.regInput[r] == a.input) {
                    a.reg = static_cast<int32_t>(r);
                }
            }
        }
    }
    // Inputs without a fixed width are VARCHAR/CHAR columns that only COUNT reads (for NULLs).
    for (size_t i = 0; i < p.inputWidths.size(); ++i) {
        if (p.inputWidths[i] == 0) {
            p.varlenInputs.push_back(static_cast<int32_t>(i));
        }
    }
    p.stateWords = word;
    p.slotWords = p.keyWords + p.stateWords;
    for (const auto &a : p.accs) {
        if ((a.kind == omg::ACC_XMIN || a.kind == omg::ACC_XMAX) && (p.slotWords & 1) != 0) {
            ++p.stateWords;  // even slots keep every slot's 16-byte states aligned
            ++p.slotWords;
            break;
        }
    }
    p.smemSlots = static_cast<int32_t>(kSmemBudget / (p.slotWords * sizeof(uint64_t)));
    p.rowsPerBatch = GetMaxRowCount(rowBytes);
    p.outContainer.assign(p.outs.size(), 0);
    for (size_t i : containerAt) {
        p.outContainer[i] = 2;
    }
    // AlignSchema columns: each output of a raw-input partial plan restated for one row.
    bool alignable = nAgg > 0 && p.dictInputs.empty() && p.varlenInputs.empty();
    for (size_t a = 0; a < nAgg; ++a) {
        const bool raw = a < inputRaws_.size() ? static_cast<bool>(inputRaws_[a]) : true;
        const bool partial = a < outputPartials_.size() ? static_cast<bool>(outputPartials_[a]) : false;
        alignable = alignable && raw && partial;
    }
    for (size_t i = 0; alignable && i < p.outs.size(); ++i) {
        const OutSpec &o = p.outs[i];
        omg::AlignCol c{};
        c.outWidth = o.outWidth;
        c.input = -1;
        switch (o.kind) {
            case omg::OUT_KEY:
                c.op = omg::ALIGN_COPY;
                c.input = p.key.cols[o.src].input;
                c.inWidth = p.key.cols[o.src].width;
                break;
            case omg::OUT_COUNT:
                // AlignSchema reads each aggregator's own input columns and ignores its mask
                // (MaskColAggregator::AlignAggSchema, mask_column_assistant_aggregator.h:75-85);
                // its batch table is built without the masks, so masked inputs read plain NULLs.
                c.op = o.countAcc < 0 || o.boundKind == 2 ? omg::ALIGN_ONE : omg::ALIGN_VALID;
                c.input = c.op == omg::ALIGN_ONE ? -1 : p.accs[o.countAcc].input;
                break;
            case omg::OUT_SUM_WRAP:
            case omg::OUT_MIN_INT:
            case omg::OUT_MAX_INT:
            case omg::OUT_SUM_DOUBLE:
            case omg::OUT_MIN_DOUBLE:
            case omg::OUT_MAX_DOUBLE:
            case omg::OUT_AVG_PARTIAL_SUM: {
                const AccSpec &acc = p.accs[o.src];
                c.op = o.kind == omg::OUT_AVG_PARTIAL_SUM
                    ? omg::ALIGN_AVG_SUM
                    : ((o.kind == omg::OUT_SUM_WRAP || o.kind == omg::OUT_MIN_INT || o.kind == omg::OUT_MAX_INT)
                              ? omg::ALIGN_INT
                              : omg::ALIGN_DOUBLE);
                c.input = acc.input;
                c.inKind = acc.inKind;
                c.inWidth = acc.inWidth;
                break;
            }
            default:
                alignable = false;
        }
        p.align.push_back(c);
    }
    if (!alignable) {
        p.align.clear();
    }
    inited_ = true;
    return OMNI_STATUS_NORMAL;
}

Operator *HashAggregationOperatorFactory::CreateOperator()
{
    Init();
    return new HashAggregationOperator(plan_, sizer_);
}

// ------------------------------------------------------------------------------ operator
namespace {
// String dictionary of one VARCHAR/CHAR group-by input (kernels/dict.cu): open-addressing
// slots (string hash, id, representative row of the batch set being inserted) and the
// characters of every id, in id order, in an arena with 64-bit offsets.  Ids are dense and
// never change, so the aggregation table keyed by ids stays valid across flushes.
struct StringDict {
    DevArray<unsigned long long> hash;
    DevArray<int32_t> id;
    DevArray<unsigned long long> rep;
    uint64_t cap = 0;
    int64_t nIds = 0;
    DevArray<int64_t> arenaOff;  // nIds + 1 entries used
    DevArray<uint8_t> arena;     // arenaBytes used
    int64_t arenaBytes = 0;
};
}  // namespace

struct HashAggregationOperator::Impl {
    omg::OpStream stream;
    omg::KernelTimer timer;
    DevArray<uint64_t> slots;
    DevArray<uint32_t> special;
    // stats[0] = groupCount, [1] = nRetry, [2] = nSpill, [3] = error
    DevArray<unsigned long long> stats;
    uint64_t capacity = 0;
    uint64_t groups = 0;
    // Batches kept for the ordered sticky-overflow path (order-dependent plans only).
    std::vector<VectorBatch *> retained;
    // Sizing, decided at the first flush: the sketch of a row sample, the group estimate used,
    // and the partition bits of the partitioned strategy (-1: global table).
    bool decided = false;
    unsigned long long sketch[omg::kSketchStats] = {};
    int64_t sketchRows = 0;  // rows of the flush the sketch sampled
    uint64_t estimate = 0;
    uint64_t plainEstimate = 0;
    bool learned = false;
    int32_t partBits = -1;
    // VARCHAR/CHAR group-by inputs: one dictionary per plan dictInputs entry.  For
    // order-dependent plans the id (and zero) columns of the retained batches stay alive
    // (retainedInputs[b]: the columns of retained batch b for dictInputs, then varlenInputs).
    std::vector<StringDict> dicts;
    std::vector<DevArray<int32_t>> keptIds;
    std::vector<std::vector<const void *>> retainedInputs;
};

HashAggregationOperator::HashAggregationOperator(const AggPlan &plan, omg::SizingModel *sizer)
    : plan_(plan), impl_(new Impl()), sizer_(sizer)
{}

HashAggregationOperator::~HashAggregationOperator()
{
    Close();
}

OmniStatus HashAggregationOperator::Close()
{
    ReleasePending();
    for (auto *b : impl_->retained) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    impl_->retained.clear();
    for (auto *b : outputs_) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    outputs_.clear();
    return OMNI_STATUS_NORMAL;
}

void HashAggregationOperator::ReleasePending()
{
    for (auto *b : pending_) {
        vec::VectorHelper::FreeVecBatch(b);
    }
    pending_.clear();
    pendingRows_ = 0;
}

int32_t HashAggregationOperator::AddInput(VectorBatch *vecBatch)
{
    hasInputedData_ = true;
    if (vecBatch == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "AddInput of a null batch", -1);
    }
    if (vecBatch->GetRowCount() <= 0) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        return 0;
    }
    for (int32_t ref : plan_.inputCols) {
        const int32_t c = ref >= omg::kFieldRefBase ? omg::FieldRefColumn(ref) : ref;  // a container's field
        if (c >= vecBatch->GetVectorCount()) {
            vec::VectorHelper::FreeVecBatch(vecBatch);
            throw OmniException("OPERATOR_RUNTIME_ERROR", "input batch lacks column " + std::to_string(c), -1);
        }
    }
    if (extracted_) {
        vec::VectorHelper::FreeVecBatch(vecBatch);
        throw OmniException("OPERATOR_RUNTIME_ERROR", "AddInput after GetOutput started", -6);
    }
    omg::FlattenTaken(vecBatch);  // dictionary-encoded vectors -> flat device vectors
    pending_.push_back(vecBatch);
    pendingRows_ += vecBatch->GetRowCount();
    if (!spillEnabled_ && pendingRows_ >= omg::AggFlushRows()) {
        Flush();
    }
    return 0;
}

omg::AggLaunch MakeAggLaunch(const AggPlan &plan, uint64_t *slots, uint64_t capacity, uint32_t *special,
    unsigned long long *stats)
{
    omg::AggLaunch p;
    std::memset(&p, 0, sizeof(p));
    p.key = plan.key;
    p.nAccs = static_cast<int32_t>(plan.accs.size());
    for (int i = 0; i < p.nAccs; ++i) {
        p.accs[i] = plan.accs[i];
    }
    p.nRegInputs = static_cast<int32_t>(plan.regInput.size());
    for (int i = 0; i < p.nRegInputs; ++i) {
        p.regInput[i] = plan.regInput[i];
        p.regWidth[i] = plan.regWidth[i];
    }
    p.stateWords = plan.stateWords;
    p.maxProbe = kGlobalMaxProbe;
    p.table.slots = slots;
    p.table.capacity = capacity;
    p.table.slotWords = plan.slotWords;
    p.table.keyWords = plan.keyWords;
    p.table.specialUsed = special;
    p.table.groupCount = stats;
    p.nRetry = stats != nullptr ? reinterpret_cast<unsigned int *>(stats + 1) : nullptr;
    p.error = stats != nullptr ? reinterpret_cast<int32_t *>(stats + 3) : nullptr;
    p.waitBudget = omg::WaitBudget();
    return p;
}

namespace {
omg::AggLaunch MakeLaunch(const AggPlan &plan, uint64_t *slots, uint64_t capacity, uint32_t *special,
    unsigned long long *stats)
{
    return MakeAggLaunch(plan, slots, capacity, special, stats);
}

constexpr int64_t kSketchMinRows = int64_t(1) << 18;  // smaller flushes: default sizing, global table
constexpr int32_t kSketchSample = 1 << 16;
constexpr double kPartLoad = 0.6;  // target load of a partition's shared table
}  // namespace

// Partition buffers of one flush (see Partition).
struct HashAggregationOperator::PartBuffers {
    std::vector<omg::BufferPtr> cols;
    std::vector<omg::BufferPtr> nulls;
    DevArray<unsigned long long> counters;  // hist then cursor
    DevArray<omg::BatchDesc> batches;
    DevArray<omg::TileDesc> tiles;
    DevArray<int32_t> tileStart;
};

VectorBatch *HashAggregationOperator::AlignSchema(VectorBatch *inputVecBatch)
{
    if (inputVecBatch == nullptr) {
        throw OmniException("INVALID_ARGUMENT", "AlignSchema of a null batch", -1);
    }
    std::unique_ptr<VectorBatch, void (*)(VectorBatch *)> in(inputVecBatch,
        [](VectorBatch *b) { vec::VectorHelper::FreeVecBatch(b); });
    if (plan_.align.empty()) {
        throw OmniException("UNSUPPORTED_ERROR",
            "AlignSchema needs every aggregator to read raw input and emit partials", -2);
    }
    const int64_t rows = inputVecBatch->GetRowCount();
    int32_t maxCol = 0;
    for (int32_t ref : plan_.inputCols) {
        maxCol = std::max(maxCol, (ref >= omg::kFieldRefBase ? omg::FieldRefColumn(ref) : ref) + 1);
    }
    if (inputVecBatch->GetVectorCount() < maxCol) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "AlignSchema batch has too few vectors", -1);
    }
    omg::RequireDevice();
    if (userStreamSet_) {
        impl_->stream.SetUser(userStream_);
    }
    cudaStream_t s = impl_->stream.Get();
    omg::FlattenDictionaries(inputVecBatch, s);
    std::vector<omg::OutColumn> cols(plan_.align.size());
    omg::BatchTable bt;
    if (rows > 0) {
        bt.Build({inputVecBatch}, plan_.inputCols);
        bt.Upload(s);
    }
    for (size_t o = 0; o < cols.size(); ++o) {
        const omg::AlignCol &c = plan_.align[o];
        omg::OutColumn &oc = cols[o];
        oc.type = plan_.outTypes[o]->GetId();
        oc.width = plan_.outTypes[o]->ByteWidth();
        oc.containerFields = o < plan_.outContainer.size() ? plan_.outContainer[o] : 0;
        const bool inContainer = (o < plan_.outContainer.size() && plan_.outContainer[o] > 0) ||
            (o > 0 && o - 1 < plan_.outContainer.size() && plan_.outContainer[o - 1] > 1);
        oc.hasNull = !inContainer && c.input >= 0 && rows > 0 && bt.AnyNulls(c.input) &&
            (c.op == omg::ALIGN_COPY || c.op == omg::ALIGN_INT || c.op == omg::ALIGN_DOUBLE);
        oc.values = omg::Buffer::NewDevice(static_cast<size_t>(rows) * oc.width + 16, s, false);
        oc.nulls = oc.hasNull ? omg::Buffer::NewDevice(omg::NullBitmapBytes(rows), s, true) : nullptr;
        if (rows > 0) {
            CudaCheck(omg::LaunchAlignColumn(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(), bt.DeviceTileOutRows(),
                          c, oc.values->Data(), oc.hasNull ? static_cast<uint8_t *>(oc.nulls->Data()) : nullptr, s),
                "align schema");
            ++counters_[0];
        }
    }
    std::vector<omg::OutColumn> outCols = cols;
    if (!deviceOutput_ && rows > 0) {
        outCols = omg::CopyColumnsToHost(cols, rows, s, 0);
        for (auto &c : outCols) {
            c.hasNull = false;  // host vectors: HasNull() scans the bitmap
        }
    }
    impl_->stream.Sync();
    if (rows == 0) {
        auto *b = new VectorBatch(0);
        for (size_t o = 0; o < cols.size(); ++o) {
            const auto &c = cols[o];
            auto empty = [](const omg::OutColumn &x) {
                return new vec::BaseVector(x.type, x.width, 0, omg::Buffer::NewHost(16, false), 0, nullptr, 0, false);
            };
            if (c.containerFields > 0) {
                std::vector<vec::BaseVector *> fields;
                for (int32_t f = 0; f < c.containerFields; ++f) {
                    fields.push_back(empty(cols[o + f]));
                }
                b->Append(new vec::BaseVector(fields));
                o += static_cast<size_t>(c.containerFields - 1);
                continue;
            }
            b->Append(empty(c));
        }
        return b;
    }
    // One batch: CarveBatches cuts at multiples of 64 rows.
    auto batches = omg::CarveBatches(outCols, rows, static_cast<int32_t>((rows + 63) / 64 * 64), 0);
    if (batches.size() != 1) {
        for (auto *b : batches) {
            vec::VectorHelper::FreeVecBatch(b);
        }
        throw OmniException("OPERATOR_RUNTIME_ERROR", "AlignSchema produced no batch", -9);
    }
    return batches[0];
}

int32_t HashAggregationOperator::GetSizingLog(int64_t *out, int32_t n) const
{
    const Impl &im = *impl_;
    std::vector<int64_t> v;
    v.push_back(im.sketchRows);
    for (int i = 0; i < omg::kSketchStats; ++i) {
        v.push_back(static_cast<int64_t>(im.sketch[i]));
    }
    v.push_back(static_cast<int64_t>(im.estimate));
    v.push_back(im.partBits);
    v.push_back(static_cast<int64_t>(std::max<uint64_t>(im.groups, uniqueKeys_)));
    v.push_back(static_cast<int64_t>(im.plainEstimate));
    v.push_back(im.learned ? 1 : 0);
    v.push_back(strategy_ == 1 ? 1 : 0);
    const int32_t m = std::min<int32_t>(n, static_cast<int32_t>(v.size()));
    for (int32_t i = 0; i < m; ++i) {
        out[i] = v[i];
    }
    return m;
}

void HashAggregationOperator::Decide(omg::BatchTable &bt, cudaStream_t s)
{
    Impl &im = *impl_;
    im.decided = true;
    const int64_t rows = bt.TotalRows();
    if (capacityHint_ > 0) {
        im.estimate = static_cast<uint64_t>(capacityHint_);  // the caller's (or a sizing model's) estimate
    } else if (sizing_ == 1 && rows > 0 && (strategy_ == 0 || strategy_ == 3)) {
        // HyperLogLog over every row's key: one pass over the keys, ~0.8% standard error.
        DevArray<unsigned int> regs(omg::kHllRegs + 2, s);
        omg::AggLaunch p = MakeLaunch(plan_, nullptr, 0, nullptr, nullptr);
        p.batches = bt.DeviceBatches();
        p.tiles = bt.DeviceTiles();
        p.nTiles = bt.NumTiles();
        CudaCheck(omg::LaunchAggHll(p, regs.Get(), s), "HyperLogLog sketch");
        ++counters_[0];
        std::vector<unsigned int> h(omg::kHllRegs + 2);
        CudaCheck(cudaMemcpyAsync(h.data(), regs.Get(), h.size() * sizeof(unsigned int), cudaMemcpyDeviceToHost, s),
            "read HyperLogLog registers");
        im.stream.Sync();
        im.sketchRows = rows;
        im.plainEstimate = omg::HllGroupEstimate(h.data(), rows);
        im.estimate = im.plainEstimate;
    } else if (rows >= kSketchMinRows && (strategy_ == 0 || strategy_ == 3)) {
        DevArray<unsigned long long> tabKeys(omg::kSketchCap, s);
        DevArray<unsigned int> tabCounts(omg::kSketchCap, s);
        DevArray<unsigned long long> st(omg::kSketchStats, s);
        omg::AggLaunch p = MakeLaunch(plan_, nullptr, 0, nullptr, nullptr);
        p.batches = bt.DeviceBatches();
        p.tiles = bt.DeviceTiles();
        p.nTiles = bt.NumTiles();
        const int32_t n = static_cast<int32_t>(std::min<int64_t>(rows, kSketchSample));
        CudaCheck(omg::LaunchAggSketch(p, n, tabKeys.Get(), tabCounts.Get(), st.Get(), s), "key sketch");
        ++counters_[0];
        CudaCheck(cudaMemcpyAsync(im.sketch, st.Get(), sizeof(im.sketch), cudaMemcpyDeviceToHost, s), "read sketch");
        im.stream.Sync();
        im.sketchRows = rows;
        im.plainEstimate = omg::PlainGroupEstimate(im.sketch, rows);
        im.estimate = im.plainEstimate;
        if (sizer_ != nullptr && sizer_->Dims()[0] == omg::kSizerFeatures) {
            int64_t log[1 + omg::kSketchStats];
            log[0] = rows;
            for (int i = 0; i < omg::kSketchStats; ++i) {
                log[1 + i] = static_cast<int64_t>(im.sketch[i]);
            }
            float x[omg::kSizerFeatures];
            float y = 0.f;
            omg::SizerFeatures(log, x);
            sizer_->Predict(x, 1, &y);
            im.estimate = omg::SizerEstimate(log, y);
            im.learned = true;
        }
    }
    // Partitions: enough that one partition's groups fill a CTA's shared table to kPartLoad.
    const bool wantPart = strategy_ == 3 || (strategy_ == 0 && rows >= kSketchMinRows);
    if (wantPart && im.estimate > 0) {
        const double perCta = kPartLoad * omg::AggPartSmemSlots(plan_.slotWords);
        const uint64_t need = NextPow2(static_cast<uint64_t>(std::ceil(static_cast<double>(im.estimate) / perCta)));
        if (need <= static_cast<uint64_t>(omg::kMaxParts) && perCta >= 1.0) {
            int bits = 0;
            while ((uint64_t(1) << bits) < need) {
                ++bits;
            }
            im.partBits = bits;
        }
    }
    if (strategy_ == 3 && im.partBits < 0) {
        im.partBits = 0;  // forced: one partition (the shared tables still sit in front of the global one)
    }
}

void HashAggregationOperator::Partition(omg::BatchTable &bt, omg::AggLaunch &p, PartBuffers &pb, cudaStream_t s)
{
    Impl &im = *impl_;
    const int32_t nParts = 1 << im.partBits;
    const int64_t rows = bt.TotalRows();
    pb.tileStart.Reset(nParts + 1, s);
    if (im.partBits == 0) {
        // One partition: the batches themselves, no copy.
        const int32_t h[2] = {0, bt.NumTiles()};
        CudaCheck(cudaMemcpyAsync(pb.tileStart.Get(), h, sizeof(h), cudaMemcpyHostToDevice, s), "partition tiles");
        im.stream.Sync();  // h is on the stack
        p.nParts = 1;
        p.partTileStart = pb.tileStart.Get();
        return;
    }
    omg::PartArgs a;
    std::memset(&a, 0, sizeof(a));
    a.partBits = im.partBits;
    a.nInputs = static_cast<int32_t>(plan_.inputCols.size());
    const int64_t capRows = rows + static_cast<int64_t>(nParts) * 64;
    for (int32_t i = 0; i < a.nInputs; ++i) {
        const int32_t w = std::max(plan_.inputWidths[i], 1);
        a.width[i] = w;
        pb.cols.push_back(omg::Buffer::NewDevice(static_cast<size_t>(capRows) * w + 16, s, false));
        a.cols[i] = pb.cols.back()->Data();
        if (bt.AnyNulls(i)) {
            pb.nulls.push_back(omg::Buffer::NewDevice(omg::NullBitmapBytes(capRows), s, true));
            a.nulls[i] = static_cast<uint32_t *>(pb.nulls.back()->Data());
        }
    }
    pb.counters.Reset(2 * static_cast<size_t>(nParts), s, true);
    a.hist = pb.counters.Get();
    a.cursor = pb.counters.Get() + nParts;
    pb.batches.Reset(nParts, s);
    a.partBatches = pb.batches.Get();
    a.maxTiles = static_cast<int32_t>(rows / omg::kTileRows + nParts + 1);
    pb.tiles.Reset(a.maxTiles, s);
    a.partTiles = pb.tiles.Get();
    a.partTileStart = pb.tileStart.Get();
    CudaCheck(omg::LaunchAggPartition(p, a, s), "hash partition");
    counters_[0] += 3;
    p.batches = pb.batches.Get();
    p.tiles = pb.tiles.Get();
    p.nTiles = a.maxTiles;
    p.nParts = nParts;
    p.partTileStart = pb.tileStart.Get();
}

namespace {
// Grow a device array to at least `need` elements (doubling), keeping its first `used`.
template <typename T> void GrowKeep(DevArray<T> &a, size_t used, size_t need, cudaStream_t s)
{
    if (a.Get() != nullptr && a.Size() >= need) {
        return;
    }
    DevArray<T> b(std::max<size_t>(need, 2 * a.Size()), s);
    if (used > 0) {
        CudaCheck(cudaMemcpyAsync(b.Get(), a.Get(), used * sizeof(T), cudaMemcpyDeviceToDevice, s), "grow array");
    }
    a = b;
}

// Insert the strings of input `input` of every row of `bt` into `d` and return each row's id
// (tile output order; 0 for NULL rows, whose key stays NULL through the column's bitmap).
DevArray<int32_t> DictEncode(StringDict &d, omg::BatchTable &bt, int32_t input, cudaStream_t s)
{
    const int64_t rows = bt.TotalRows();
    DevArray<int32_t> err(1, s, true);
    // At most half full after this batch set, even if every row brings a new string.
    const uint64_t need = NextPow2(std::max<uint64_t>(1024, 2 * static_cast<uint64_t>(d.nIds + rows)));
    if (need > d.cap) {
        DevArray<unsigned long long> hash(need, s);
        DevArray<int32_t> id(need, s);
        CudaCheck(cudaMemsetAsync(hash.Get(), 0xff, need * sizeof(unsigned long long), s), "init dictionary");
        CudaCheck(cudaMemsetAsync(id.Get(), 0xff, need * sizeof(int32_t), s), "init dictionary");
        if (d.cap > 0) {
            CudaCheck(omg::LaunchDictRehash(d.hash.Get(), d.id.Get(), d.cap, hash.Get(), id.Get(), need, err.Get(), s),
                "grow dictionary");
        }
        d.hash = hash;
        d.id = id;
        d.rep.Reset(need, s);
        d.cap = need;
    }
    if (d.arenaOff.Get() == nullptr) {
        d.arenaOff.Reset(1024, s, true);
        d.arena.Reset(4096, s);
    }
    CudaCheck(cudaMemsetAsync(d.rep.Get(), 0xff, d.cap * sizeof(unsigned long long), s), "reset dictionary");
    DevArray<int32_t> rowSlot(static_cast<size_t>(rows), s);
    CudaCheck(omg::LaunchDictInsert(bt.DeviceBatches(), bt.DeviceTiles(), bt.NumTiles(), bt.DeviceTileOutRows(), input,
                  d.hash.Get(), d.id.Get(), d.rep.Get(), d.cap, d.arenaOff.Get(), d.arena.Get(), rowSlot.Get(),
                  err.Get(), s),
        "dictionary insert");
    const size_t maxNew = static_cast<size_t>(std::min<uint64_t>(static_cast<uint64_t>(rows), d.cap));
    DevArray<unsigned int> counter(1, s, true);
    DevArray<unsigned long long> newRep(maxNew, s);
    DevArray<uint32_t> newLen(maxNew, s);
    CudaCheck(omg::LaunchDictMaterialize(d.hash.Get(), d.id.Get(), d.rep.Get(), d.cap, static_cast<int32_t>(d.nIds),
                  counter.Get(), newRep.Get(), newLen.Get(), bt.DeviceBatches(), input, s),
        "dictionary ids");
    unsigned int h[2] = {0, 0};
    CudaCheck(cudaMemcpyAsync(h, counter.Get(), sizeof(unsigned int), cudaMemcpyDeviceToHost, s), "read new ids");
    CudaCheck(cudaMemcpyAsync(h + 1, err.Get(), sizeof(int32_t), cudaMemcpyDeviceToHost, s), "read new ids");
    CudaCheck(cudaStreamSynchronize(s), "read new ids");
    if (h[1] != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "string dictionary overflow", -9);
    }
    const int64_t nNew = h[0];
    if (d.nIds + nNew >= (int64_t(1) << 31)) {
        throw OmniException("UNSUPPORTED_ERROR", "more than 2^31 distinct strings in one group-by column", -2);
    }
    if (nNew > 0) {
        DevArray<int64_t> offs;
        const int64_t bytes = omg::ScanLengths(newLen.Get(), nNew, offs, s);
        GrowKeep(d.arenaOff, static_cast<size_t>(d.nIds + 1), static_cast<size_t>(d.nIds + nNew + 1), s);
        CudaCheck(omg::LaunchDictShiftOffsets(offs.Get(), nNew, d.arenaBytes, d.arenaOff.Get() + d.nIds, s),
            "dictionary offsets");
        GrowKeep(d.arena, static_cast<size_t>(d.arenaBytes), static_cast<size_t>(d.arenaBytes + bytes + 16), s);
        CudaCheck(omg::LaunchDictAppend(newRep.Get(), nNew, static_cast<int32_t>(d.nIds), d.arenaOff.Get(),
                      d.arena.Get(), bt.DeviceBatches(), input, s),
            "dictionary characters");
        d.nIds += nNew;
        d.arenaBytes += bytes;
    }
    DevArray<int32_t> ids(static_cast<size_t>(rows), s);
    CudaCheck(omg::LaunchDictRowIds(rowSlot.Get(), rows, d.id.Get(), ids.Get(), s), "row ids");
    return ids;
}
}  // namespace

// The string dictionaries SMIN/SMAX compare through (their arenas move when they grow, so a
// launch binds them after the batch set was encoded).
void HashAggregationOperator::BindStrings(omg::AggLaunch &p) const
{
    const Impl &im = *impl_;
    for (size_t j = 0; j < plan_.dictInputs.size() && j < im.dicts.size(); ++j) {
        p.strOff[plan_.dictInputs[j]] = im.dicts[j].arenaOff.Get();
        p.strChars[plan_.dictInputs[j]] = im.dicts[j].arena.Get();
    }
}

// VARCHAR/CHAR inputs of a batch set: group-by columns become dictionary ids, COUNT-only
// columns a zero byte per row (their NULL bitmaps stay the batches' own); the batch
// descriptors are uploaded again.
void HashAggregationOperator::EncodeStrings(omg::BatchTable &bt, cudaStream_t s)
{
    Impl &im = *impl_;
    const size_t nb = bt.NumBatches();
    std::vector<std::vector<const void *>> perBatch(nb);
    im.dicts.resize(plan_.dictInputs.size());
    for (size_t j = 0; j < plan_.dictInputs.size(); ++j) {
        DevArray<int32_t> ids = DictEncode(im.dicts[j], bt, plan_.dictInputs[j], s);
        for (size_t b = 0; b < nb; ++b) {
            const int32_t *p = ids.Get() + bt.BatchRowBase(b);
            bt.SetInput(b, plan_.dictInputs[j], p);
            perBatch[b].push_back(p);
        }
        im.keptIds.push_back(ids);
    }
    if (!plan_.varlenInputs.empty()) {
        DevArray<int32_t> zeros(static_cast<size_t>(bt.TotalRows() + 16) / 4 + 1, s, true);
        for (size_t b = 0; b < nb; ++b) {
            const uint8_t *p = reinterpret_cast<const uint8_t *>(zeros.Get()) + bt.BatchRowBase(b);
            for (int32_t in : plan_.varlenInputs) {
                bt.SetInput(b, in, p);
                perBatch[b].push_back(p);
            }
        }
        im.keptIds.push_back(zeros);
    }
    bt.Upload(s);
    if (plan_.orderDependent) {
        for (auto &v : perBatch) {
            im.retainedInputs.push_back(v);
        }
    }
}

void HashAggregationOperator::Flush()
{
    if (pending_.empty()) {
        return;
    }
    omg::RequireDevice();
    Impl &im = *impl_;
    if (userStreamSet_) {
        im.stream.SetUser(userStream_);
    }
    cudaStream_t s = im.stream.Get();
    if (im.stats.Get() == nullptr) {
        im.stats.Reset(8, s, true);
    }
    omg::BatchTable bt;
    bt.Build(pending_, plan_.inputCols, omg::kTileRows, &plan_.inputMasks);
    bt.Upload(s);
    const int64_t rows = bt.TotalRows();
    if (!plan_.dictInputs.empty() || !plan_.varlenInputs.empty()) {
        EncodeStrings(bt, s);
    }
    if (!im.decided) {
        Decide(bt, s);
    }
    // Create the table on first use, sized for the group estimate (load factor <= 1/2).
    if (im.capacity == 0) {
        uint64_t cap = im.estimate > 0 ? NextPow2(im.estimate * 2) : kDefaultCapacity;
        cap = std::max<uint64_t>(cap, 1024);
        im.slots.Reset((cap + 2) * plan_.slotWords, s);
        im.special.Reset(2, s, true);
        im.capacity = cap;
        omg::AggLaunch init = MakeLaunch(plan_, im.slots.Get(), cap, im.special.Get(), im.stats.Get());
        CudaCheck(omg::LaunchAggInitTable(init, s), "init aggregation table");
        ++counters_[0];
    }
    const int sms = omg::DeviceSMCount();
    int smemSlots = 0;
    // GLOBAL (2): global table only.  SMEM (1): a per-CTA shared table in front of the global
    // one.  PARTITIONED (3, or AUTO when the estimate says the groups fit): rows are hash
    // partitioned so that each CTA's shared table holds one partition's groups.
    if (strategy_ == 1) {  // OMG_AGG_STRATEGY_SMEM
        smemSlots = plan_.smemSlots;
    }
    const int grid = 0;  // the launcher fills every SM to its occupancy limit
    const int maxGrid = sms * 4;
    // Partition buffers live until the retries (which address rows of the partitions) are done.
    PartBuffers part;
    const omg::BatchDesc *rowBatches = bt.DeviceBatches();
    DevArray<unsigned long long> retryA(static_cast<size_t>(rows), s);
    DevArray<unsigned long long> retryB;
    omg::AggLaunch p = MakeLaunch(plan_, im.slots.Get(), im.capacity, im.special.Get(), im.stats.Get());
    BindStrings(p);
    p.batches = bt.DeviceBatches();
    p.tiles = bt.DeviceTiles();
    p.nTiles = bt.NumTiles();
    if (im.partBits >= 0) {
        smemSlots = omg::AggPartSmemSlots(plan_.slotWords);
        Partition(bt, p, part, s);
        rowBatches = p.batches;
    }
    const size_t spillCap = static_cast<size_t>(smemSlots) * maxGrid;
    DevArray<uint64_t> spillA(std::max<size_t>(spillCap, 1) * plan_.slotWords, s);
    DevArray<uint64_t> spillB;
    CudaCheck(cudaMemsetAsync(im.stats.Get() + 1, 0, 3 * sizeof(unsigned long long), s), "reset stats");
    p.retry = retryA.Get();
    p.retryCap = static_cast<uint32_t>(rows);
    p.smemSlots = smemSlots;
    unsigned int *nSpill = reinterpret_cast<unsigned int *>(im.stats.Get() + 2);
    im.timer.Start(s);
    CudaCheck(omg::LaunchAgg(p, spillA.Get(), nSpill, static_cast<uint32_t>(spillCap), nullptr, 0, grid, s),
        "aggregation kernel");
    im.timer.Stop(s);
    ++counters_[0];
    unsigned long long h[4];
    CudaCheck(cudaMemcpyAsync(h, im.stats.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read stats");
    im.stream.Sync();
    counters_[6] += im.timer.ElapsedNs();
    ++counters_[7];
    uint64_t nRetry = static_cast<unsigned int>(h[1]);
    uint64_t nSpillH = static_cast<unsigned int>(h[2]);
    int32_t err = static_cast<int32_t>(h[3]);
    if (err != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "aggregation kernel error " + std::to_string(err),
            err == 7 ? -7 : -9);
    }
    im.groups = h[0];
    // Exact resize path: grow the table and re-run the rows (and partial states) that could
    // not be placed.  Each round at least doubles the capacity.
    while (nRetry > 0 || nSpillH > 0) {
        const uint64_t need = NextPow2(std::max<uint64_t>(im.capacity * 2, 2 * (im.groups + nRetry + nSpillH)));
        DevArray<uint64_t> newSlots((need + 2) * plan_.slotWords, s);
        DevArray<uint32_t> newSpecial(2, s, true);
        omg::AggLaunch to = MakeLaunch(plan_, newSlots.Get(), need, newSpecial.Get(), im.stats.Get());
        CudaCheck(omg::LaunchAggInitTable(to, s), "init grown table");
        omg::AggLaunch from = MakeLaunch(plan_, im.slots.Get(), im.capacity, im.special.Get(), im.stats.Get());
        CudaCheck(omg::LaunchAggRehash(to, from.table, to.table, s), "rehash");
        im.slots = newSlots;
        im.special = newSpecial;
        im.capacity = need;
        ++counters_[1];
        counters_[2] += static_cast<int64_t>(nRetry);
        retryB.Reset(std::max<uint64_t>(nRetry, 1), s);
        spillB.Reset(std::max<uint64_t>(nSpillH, 1) * plan_.slotWords, s);
        CudaCheck(cudaMemsetAsync(im.stats.Get() + 1, 0, 3 * sizeof(unsigned long long), s), "reset stats");
        omg::AggLaunch r = MakeLaunch(plan_, im.slots.Get(), im.capacity, im.special.Get(), im.stats.Get());
        BindStrings(r);
        r.batches = rowBatches;
        r.retry = retryB.Get();
        r.retryCap = static_cast<uint32_t>(std::max<uint64_t>(nRetry, 1));
        r.retryIn = retryA.Get();
        r.nRetryIn = static_cast<uint32_t>(nRetry);
        const int rgrid = static_cast<int>(std::min<uint64_t>((nRetry + nSpillH + 511) / 512 + 1, sms * 8ull));
        CudaCheck(omg::LaunchAgg(r, spillB.Get(), nSpill, static_cast<uint32_t>(std::max<uint64_t>(nSpillH, 1)),
                      spillA.Get(), static_cast<uint32_t>(nSpillH), rgrid, s),
            "aggregation retry kernel");
        ++counters_[0];
        CudaCheck(cudaMemcpyAsync(h, im.stats.Get(), sizeof(h), cudaMemcpyDeviceToHost, s), "read stats");
        im.stream.Sync();
        std::swap(retryA, retryB);
        std::swap(spillA, spillB);
        nRetry = static_cast<unsigned int>(h[1]);
        nSpillH = static_cast<unsigned int>(h[2]);
        err = static_cast<int32_t>(h[3]);
        im.groups = h[0];
        if (err != 0) {
            throw OmniException("OPERATOR_RUNTIME_ERROR", "aggregation retry error " + std::to_string(err), -9);
        }
    }
    // Keep the load factor under one half for the next batches (the reference grows x4).
    if (im.groups * 2 > im.capacity) {
        const uint64_t need = NextPow2(im.groups * 4);
        DevArray<uint64_t> newSlots((need + 2) * plan_.slotWords, s);
        DevArray<uint32_t> newSpecial(2, s, true);
        omg::AggLaunch to = MakeLaunch(plan_, newSlots.Get(), need, newSpecial.Get(), im.stats.Get());
        CudaCheck(omg::LaunchAggInitTable(to, s), "init grown table");
        omg::AggLaunch from = MakeLaunch(plan_, im.slots.Get(), im.capacity, im.special.Get(), im.stats.Get());
        CudaCheck(omg::LaunchAggRehash(to, from.table, to.table, s), "rehash");
        im.slots = newSlots;
        im.special = newSpecial;
        im.capacity = need;
        ++counters_[1];
        im.stream.Sync();
    }
    counters_[3] = static_cast<int64_t>(im.groups);
    if (!plan_.orderDependent) {
        im.keptIds.clear();  // freed stream-ordered, after the kernels that read them
    }
    if (plan_.orderDependent) {
        for (auto *b : pending_) {
            im.retained.push_back(b);
        }
        pending_.clear();
        pendingRows_ = 0;
    } else {
        ReleasePending();
    }
}

// VARCHAR/CHAR key and MIN/MAX columns of the extracted groups: dictionary ids back to strings
// (lengths, a scan to offsets, then the characters), on the device.
void HashAggregationOperator::DecodeStrings(std::vector<omg::OutColumn> &cols, int64_t rows, cudaStream_t s)
{
    Impl &im = *impl_;
    for (size_t o = 0; o < plan_.outs.size(); ++o) {
        const OutSpec &os = plan_.outs[o];
        if ((os.kind != omg::OUT_KEY && os.kind != omg::OUT_STR_ID) || !IsVarlen(plan_.outTypes[o]->GetId())) {
            continue;
        }
        const int32_t input = os.kind == omg::OUT_KEY ? plan_.key.cols[os.src].input : plan_.accs[os.src].input;
        const size_t j = static_cast<size_t>(
            std::find(plan_.dictInputs.begin(), plan_.dictInputs.end(), input) - plan_.dictInputs.begin());
        StringDict &d = im.dicts.at(j);
        omg::OutColumn &c = cols[o];
        const int32_t *ids = static_cast<const int32_t *>(c.values->Data());
        const uint8_t *nulls = static_cast<const uint8_t *>(c.nulls->Data());
        DevArray<uint32_t> lens(static_cast<size_t>(rows), s);
        CudaCheck(omg::LaunchDictDecodeLens(ids, nulls, rows, d.arenaOff.Get(), lens.Get(), s), "key string lengths");
        DevArray<int64_t> offs64;
        const int64_t total = omg::ScanLengths(lens.Get(), rows, offs64, s);
        if (total >= (int64_t(1) << 31)) {
            throw OmniException("UNSUPPORTED_ERROR", "more than 2 GiB of VARCHAR group-by keys in the output", -2);
        }
        omg::BufferPtr chars = omg::Buffer::NewDevice(static_cast<size_t>(total) + 16, s, false);
        omg::BufferPtr offs32 = omg::Buffer::NewDevice((static_cast<size_t>(rows) + 1) * sizeof(int32_t), s, false);
        CudaCheck(omg::LaunchDictDecodeCopy(ids, nulls, rows, d.arenaOff.Get(), d.arena.Get(), offs64.Get(),
                      static_cast<uint8_t *>(chars->Data()), static_cast<int32_t *>(offs32->Data()), total, s),
            "key strings");
        ++counters_[0];
        c.width = 0;
        c.values = chars;
        c.offsets = offs32;
        c.dataBytes = total;
    }
}

// A spilled partition's output batch (device) with the id columns `outs` turned back into
// VARCHAR/CHAR vectors through this operator's dictionaries; copied to the host unless the
// operator outputs device vectors.  Takes the batch, returns the result.
VectorBatch *HashAggregationOperator::DecodeKeyIds(VectorBatch *batch, const std::vector<size_t> &outs, cudaStream_t s)
{
    Impl &im = *impl_;
    std::unique_ptr<VectorBatch, void (*)(VectorBatch *)> b(batch, [](VectorBatch *x) { vec::VectorHelper::FreeVecBatch(x); });
    const int64_t rows = b->GetRowCount();
    for (size_t o : outs) {
        const OutSpec &os = plan_.outs[o];
        const int32_t input = plan_.key.cols[os.src].input;
        const size_t j = static_cast<size_t>(
            std::find(plan_.dictInputs.begin(), plan_.dictInputs.end(), input) - plan_.dictInputs.begin());
        StringDict &d = im.dicts.at(j);
        vec::BaseVector *v = b->Get(static_cast<int32_t>(o));
        const int32_t *ids = reinterpret_cast<const int32_t *>(v->RawValues());
        const uint8_t *nulls = v->NullFlag() ? v->RawNulls() : nullptr;
        DevArray<uint32_t> lens(static_cast<size_t>(std::max<int64_t>(rows, 1)), s);
        CudaCheck(omg::LaunchDictDecodeLens(ids, nulls, rows, d.arenaOff.Get(), lens.Get(), s), "key string lengths");
        DevArray<int64_t> offs64;
        const int64_t total = omg::ScanLengths(lens.Get(), rows, offs64, s);
        if (total >= (int64_t(1) << 31)) {
            throw OmniException("UNSUPPORTED_ERROR", "more than 2 GiB of VARCHAR group-by keys in one output batch", -2);
        }
        omg::BufferPtr chars = omg::Buffer::NewDevice(static_cast<size_t>(total) + 16, s, false);
        omg::BufferPtr offs32 = omg::Buffer::NewDevice((static_cast<size_t>(rows) + 1) * sizeof(int32_t), s, false);
        CudaCheck(omg::LaunchDictDecodeCopy(ids, nulls, rows, d.arenaOff.Get(), d.arena.Get(), offs64.Get(),
                      static_cast<uint8_t *>(chars->Data()), static_cast<int32_t *>(offs32->Data()), total, s),
            "key strings");
        ++counters_[0];
        im.stream.Sync();  // lens / offs64 are freed on return
        b->Set(static_cast<int32_t>(o), new vec::BaseVector(plan_.outTypes[o]->GetId(), static_cast<int32_t>(rows), chars,
                                            total, offs32, 0, v->NullsBufferPtr(), v->NullsOffset(), v->NullFlag()));
    }
    if (deviceOutput_) {
        return b.release();
    }
    VectorBatch *h = vec::VectorHelper::CopyBatch(b.get(), false, s);
    for (int32_t i = 0; i < h->GetVectorCount(); ++i) {
        h->Get(i)->SetNullFlag(false);  // host vectors: HasNull() scans the bitmap
    }
    return h;
}

void HashAggregationOperator::SetSpill(bool enabled, uint64_t deviceBudgetBytes)
{
    bool strAgg = !plan_.varlenInputs.empty();
    for (const auto &o : plan_.outs) {
        strAgg = strAgg || o.kind == omg::OUT_STR_ID;
    }
    if (enabled && strAgg) {
        throw OmniException("UNSUPPORTED_ERROR",
            "spill takes VARCHAR/CHAR group-by keys but not MIN/MAX or COUNT of VARCHAR/CHAR values", -2);
    }
    if (enabled && deviceBudgetBytes == 0) {
        throw OmniException("INVALID_ARGUMENT", "spill needs a device memory budget", -1);
    }
    if (enabled && impl_->capacity != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "spill must be enabled before input is aggregated", -6);
    }
    spillEnabled_ = enabled;
    spillBudget_ = deviceBudgetBytes;
}

namespace {
constexpr int kMaxSpillBits = 6;  // up to 64 partitions
}

// Spill path: when the estimated group table of all staged rows exceeds the budget, the rows are
// hash-partitioned (the partitioned strategy's kernels, with pinned host memory as the target,
// written by the GPU directly) and each partition is aggregated by its own operator of the same
// plan, one at a time, so the device holds one partition's table.  Returns false when everything
// fits (the ordinary path then runs).
bool HashAggregationOperator::ExtractSpilled()
{
    if (pending_.empty()) {
        return false;
    }
    omg::RequireDevice();
    Impl &im = *impl_;
    if (userStreamSet_) {
        im.stream.SetUser(userStream_);
    }
    cudaStream_t s = im.stream.Get();
    if (im.stats.Get() == nullptr) {
        im.stats.Reset(8, s, true);
    }
    const size_t slotBytes = static_cast<size_t>(plan_.slotWords) * sizeof(uint64_t);
    uint64_t estimate = 0;
    // VARCHAR/CHAR keys: every pending row's string goes into this operator's dictionaries once;
    // the partitions carry the int32 ids and the partitions' key ids come back as strings.
    std::map<const VectorBatch *, std::vector<const void *>> idsOf;
    {
        omg::BatchTable bt;
        bt.Build(pending_, plan_.inputCols, omg::kTileRows, &plan_.inputMasks);
        bt.Upload(s);
        if (!plan_.dictInputs.empty()) {
            EncodeStrings(bt, s);
            const size_t nIds = plan_.dictInputs.size();
            for (size_t b = 0; b < pending_.size(); ++b) {
                std::vector<const void *> &v = idsOf[pending_[b]];
                for (size_t j = 0; j < nIds; ++j) {
                    const omg::DevArray<int32_t> &ids = im.keptIds[im.keptIds.size() - nIds + j];
                    v.push_back(ids.Get() + bt.BatchRowBase(b));
                }
            }
        }
        if (!im.decided) {
            Decide(bt, s);
        }
        estimate = im.estimate > 0 ? im.estimate : static_cast<uint64_t>(bt.TotalRows());
        im.stream.Sync();
    }
    const double need = 2.0 * static_cast<double>(estimate) * static_cast<double>(slotBytes);  // load <= 1/2
    if (need <= static_cast<double>(spillBudget_)) {
        return false;
    }
    int bits = 1;
    while (bits < kMaxSpillBits && need / static_cast<double>(1 << bits) > static_cast<double>(spillBudget_)) {
        ++bits;
    }
    const int32_t nParts = 1 << bits;
    // A partition batch holds one column per kernel input (values and NULLs as the kernels read
    // them, masks applied), and the partitions are aggregated by a plan reading input i from
    // column i without masks.
    const int32_t nInputs = static_cast<int32_t>(plan_.inputCols.size());
    std::vector<DataTypeId> colType(static_cast<size_t>(nInputs), OMNI_BYTE);
    for (int32_t i = 0; i < nInputs; ++i) {
        const int32_t c = plan_.inputCols[i];
        const vec::BaseVector *v = c >= omg::kFieldRefBase
            ? pending_.front()->Get(omg::FieldRefColumn(c))->Field(omg::FieldRefField(c))
            : pending_.front()->Get(c);
        colType[static_cast<size_t>(i)] = v->GetTypeId();
    }
    AggPlan partPlan = plan_;
    for (int32_t i = 0; i < nInputs; ++i) {
        partPlan.inputCols[i] = i;
        partPlan.inputMasks[i] = -1;
        if (std::find(plan_.dictInputs.begin(), plan_.dictInputs.end(), i) != plan_.dictInputs.end()) {
            colType[static_cast<size_t>(i)] = OMNI_INT;  // string ids
        }
    }
    // The partitions aggregate the key ids as INT keys; the ids become strings afterwards.
    partPlan.dictInputs.clear();
    std::vector<size_t> strKeyOuts;
    for (size_t o = 0; o < partPlan.outs.size(); ++o) {
        if (partPlan.outs[o].kind == omg::OUT_KEY && IsVarlen(plan_.outTypes[o]->GetId())) {
            partPlan.outTypes[o] = IntType();
            strKeyOuts.push_back(o);
        }
    }
    std::vector<std::vector<VectorBatch *>> parts(static_cast<size_t>(nParts));
    const int64_t chunkRows = omg::AggFlushRows();
    size_t next = 0;
    try {
        while (next < pending_.size()) {
            std::vector<VectorBatch *> chunk;
            int64_t rows = 0;
            while (next < pending_.size() && (chunk.empty() || rows + pending_[next]->GetRowCount() <= chunkRows)) {
                rows += pending_[next]->GetRowCount();
                chunk.push_back(pending_[next++]);
            }
            omg::BatchTable bt;
            bt.Build(chunk, plan_.inputCols, omg::kTileRows, &plan_.inputMasks);
            for (size_t b = 0; b < chunk.size() && !plan_.dictInputs.empty(); ++b) {
                const std::vector<const void *> &v = idsOf.at(chunk[b]);
                for (size_t j = 0; j < plan_.dictInputs.size(); ++j) {
                    bt.SetInput(b, plan_.dictInputs[j], v[j]);
                }
            }
            bt.Upload(s);
            omg::AggLaunch p = MakeLaunch(plan_, nullptr, 0, nullptr, nullptr);
            p.batches = bt.DeviceBatches();
            p.tiles = bt.DeviceTiles();
            p.nTiles = bt.NumTiles();
            omg::PartArgs a;
            std::memset(&a, 0, sizeof(a));
            a.partBits = bits;
            a.nInputs = static_cast<int32_t>(plan_.inputCols.size());
            const int64_t capRows = rows + static_cast<int64_t>(nParts) * 64;
            std::vector<omg::BufferPtr> hostCols(static_cast<size_t>(a.nInputs));
            std::vector<omg::BufferPtr> hostNulls(static_cast<size_t>(a.nInputs));
            for (int32_t i = 0; i < a.nInputs; ++i) {
                const int32_t w = std::max(plan_.inputWidths[i], 1);
                a.width[i] = w;
                hostCols[i] = omg::Buffer::NewHost(static_cast<size_t>(capRows) * w + 16, false);
                a.cols[i] = hostCols[i]->Data();
                spilledBytes_ += static_cast<uint64_t>(rows) * static_cast<uint64_t>(w);
                if (bt.AnyNulls(i)) {
                    hostNulls[i] = omg::Buffer::NewHost(omg::NullBitmapBytes(capRows), true);
                    a.nulls[i] = static_cast<uint32_t *>(hostNulls[i]->Data());
                    spilledBytes_ += static_cast<uint64_t>(rows + 7) / 8;
                }
            }
            DevArray<unsigned long long> counters(2 * static_cast<size_t>(nParts), s, true);
            a.hist = counters.Get();
            a.cursor = counters.Get() + nParts;
            // Plans whose results depend on row order (sticky-overflow sums resolved by the
            // ordered replay) keep the input order of each group's rows in its partition.
            DevArray<unsigned int> tileHist;
            if (plan_.orderDependent) {
                tileHist.Reset(static_cast<size_t>(std::max(bt.NumTiles(), 1)) * static_cast<size_t>(nParts), s);
                a.stable = 1;
                a.tileHist = tileHist.Get();
            }
            DevArray<omg::BatchDesc> partBatches(static_cast<size_t>(nParts), s);
            a.partBatches = partBatches.Get();
            a.maxTiles = static_cast<int32_t>(rows / omg::kTileRows + nParts + 1);
            DevArray<omg::TileDesc> tiles(static_cast<size_t>(a.maxTiles), s);
            DevArray<int32_t> tileStart(static_cast<size_t>(nParts) + 1, s);
            a.partTiles = tiles.Get();
            a.partTileStart = tileStart.Get();
            CudaCheck(omg::LaunchAggPartition(p, a, s), "spill partition");
            counters_[0] += 3;
            std::vector<omg::BatchDesc> desc(static_cast<size_t>(nParts));
            CudaCheck(cudaMemcpyAsync(desc.data(), partBatches.Get(), sizeof(omg::BatchDesc) * nParts,
                          cudaMemcpyDeviceToHost, s),
                "read spill partitions");
            im.stream.Sync();
            for (int32_t q = 0; q < nParts; ++q) {
                const int64_t n = desc[q].rows;
                const int64_t base = desc[q].rowBase;  // a multiple of 64 rows
                if (n == 0) {
                    continue;
                }
                auto *vb = new VectorBatch(static_cast<size_t>(n));
                for (int32_t i = 0; i < nInputs; ++i) {
                    const int32_t w = a.width[i];
                    vb->Append(new vec::BaseVector(colType[static_cast<size_t>(i)], w, static_cast<int32_t>(n), hostCols[i],
                        static_cast<size_t>(base) * w, hostNulls[i], static_cast<size_t>(base / 8),
                        hostNulls[i] != nullptr));
                }
                parts[static_cast<size_t>(q)].push_back(vb);
            }
        }
    } catch (...) {
        for (auto &pl : parts) {
            for (auto *b : pl) {
                vec::VectorHelper::FreeVecBatch(b);
            }
        }
        throw;
    }
    ReleasePending();
    // One operator of the same plan per partition; its output batches become this operator's.
    uniqueKeys_ = 0;
    for (auto &pl : parts) {
        if (pl.empty()) {
            continue;
        }
        HashAggregationOperator part(partPlan, sizer_);
        part.SetStrategy(strategy_, 0);
        // String keys are decoded on the device: the partition's output stays there until then.
        part.SetDeviceOutput(deviceOutput_ || !strKeyOuts.empty());
        if (userStreamSet_) {
            part.SetStream(userStream_);
        }
        size_t k = 0;
        try {
            for (; k < pl.size(); ++k) {
                part.AddInput(pl[k]);
            }
        } catch (...) {
            for (++k; k < pl.size(); ++k) {
                vec::VectorHelper::FreeVecBatch(pl[k]);
            }
            throw;
        }
        VectorBatch *out = nullptr;
        while (part.GetOutput(&out) != 0 && out != nullptr) {
            if (!strKeyOuts.empty()) {
                out = DecodeKeyIds(out, strKeyOuts, s);
            }
            outputs_.push_back(out);
            counters_[5] += out->GetRowCount();
            out = nullptr;
        }
        uniqueKeys_ += part.GetHashMapUniqueKeys();
        counters_[0] += part.Counters()[0];
        counters_[6] += part.Counters()[6];
        counters_[7] += part.Counters()[7];
    }
    counters_[3] = static_cast<int64_t>(uniqueKeys_);
    return true;
}

void HashAggregationOperator::Extract()
{
    if (spillEnabled_ && ExtractSpilled()) {
        return;
    }
    Flush();
    Impl &im = *impl_;
    if (im.capacity == 0) {
        uniqueKeys_ = 0;
        return;
    }
    if (userStreamSet_) {
        im.stream.SetUser(userStream_);
    }
    cudaStream_t s = im.stream.Get();
    omg::AggLaunch base = MakeLaunch(plan_, im.slots.Get(), im.capacity, im.special.Get(), im.stats.Get());
    DevArray<unsigned long long> cnt(4, s, true);
    CudaCheck(omg::LaunchAggCount(base.table, plan_.key.kind, cnt.Get(), s), "count groups");
    unsigned long long nGroups = 0;
    CudaCheck(cudaMemcpyAsync(&nGroups, cnt.Get(), sizeof(nGroups), cudaMemcpyDeviceToHost, s), "read group count");
    im.stream.Sync();
    uniqueKeys_ = nGroups;
    counters_[3] = static_cast<int64_t>(nGroups);
    if (nGroups == 0) {
        return;
    }
    const size_t nOut = plan_.outs.size();
    std::vector<omg::OutColumn> cols(nOut);
    for (size_t o = 0; o < nOut; ++o) {
        const OutSpec &os = plan_.outs[o];
        cols[o].type = plan_.outTypes[o]->GetId();
        cols[o].width = os.outWidth;
        cols[o].values = omg::Buffer::NewDevice(static_cast<size_t>(nGroups) * os.outWidth + 16, s, false);
        cols[o].nulls = omg::Buffer::NewDevice(omg::NullBitmapBytes(static_cast<int64_t>(nGroups)), s, true);
        cols[o].hasNull = os.kind != omg::OUT_COUNT && os.kind != omg::OUT_IS_EMPTY;
    }
    for (size_t o = 0; o < nOut && o < plan_.outContainer.size(); ++o) {
        // A container's fields (a partial AVG's sum and count) are never NULL.
        cols[o].containerFields = plan_.outContainer[o];
        for (int32_t f = 0; f < plan_.outContainer[o]; ++f) {
            cols[o + f].hasNull = false;
        }
    }
    omg::AggExtract e;
    std::memset(&e, 0, sizeof(e));
    e.table = base.table;
    e.key = plan_.key;
    e.nAccs = static_cast<int32_t>(plan_.accs.size());
    for (int i = 0; i < e.nAccs; ++i) {
        e.accs[i] = plan_.accs[i];
    }
    e.nOut = static_cast<int32_t>(nOut);
    for (size_t o = 0; o < nOut; ++o) {
        e.out[o] = plan_.outs[o];
        e.out[o].values = cols[o].values->Data();
        e.out[o].nulls = static_cast<uint8_t *>(cols[o].nulls->Data());
    }
    e.overflowAsNull = plan_.overflowAsNull ? 1 : 0;
    // cnt[0] = nGroups (reused as outCount after reset), cnt[1] = error, cnt[2] = nAmbiguous
    const uint32_t ambCap = static_cast<uint32_t>(std::min<unsigned long long>(nGroups, 1ull << 22));
    DevArray<unsigned long long> ambSlots(ambCap, s);
    CudaCheck(cudaMemsetAsync(cnt.Get(), 0, 4 * sizeof(unsigned long long), s), "reset counters");
    e.outCount = cnt.Get();
    e.error = reinterpret_cast<int32_t *>(cnt.Get() + 1);
    e.nAmbiguous = cnt.Get() + 2;
    e.ambiguousSlots = ambSlots.Get();
    e.ambiguousCap = ambCap;
    CudaCheck(omg::LaunchAggExtract(e, s), "extract groups");
    ++counters_[0];
    unsigned long long hc[4];
    CudaCheck(cudaMemcpyAsync(hc, cnt.Get(), sizeof(hc), cudaMemcpyDeviceToHost, s), "read extract counters");
    im.stream.Sync();
    if (hc[2] > 0) {
        // Some groups' sticky-overflow outcome depends on row order: replay those groups in
        // arrival order over the retained batches, then extract again with the answers.
        if (hc[2] > ambCap) {
            throw OmniException("UNSUPPORTED_ERROR", "too many order-dependent overflow groups", -2);
        }
        counters_[4] = static_cast<int64_t>(hc[2]);
        omg::BatchTable bt;
        bt.Build(im.retained, plan_.inputCols, 1 << 30, &plan_.inputMasks);
        // VARCHAR inputs read through the id / zero columns their flush made (same order).
        const size_t nDict = plan_.dictInputs.size();
        for (size_t b = 0; b < im.retainedInputs.size() && b < bt.NumBatches(); ++b) {
            for (size_t j = 0; j < im.retainedInputs[b].size(); ++j) {
                const int32_t in = j < nDict ? plan_.dictInputs[j] : plan_.varlenInputs[j - nDict];
                bt.SetInput(b, in, im.retainedInputs[b][j]);
            }
        }
        bt.Upload(s);
        DevArray<uint8_t> forced(im.capacity + 2, s, true);
        omg::AggLaunch p = base;
        BindStrings(p);
        p.batches = bt.DeviceBatches();
        CudaCheck(omg::LaunchAggOrdered(p, static_cast<int32_t>(im.retained.size()), e, ambSlots.Get(),
                      static_cast<uint32_t>(hc[2]), forced.Get(), s),
            "ordered overflow replay");
        for (size_t o = 0; o < nOut; ++o) {
            CudaCheck(cudaMemsetAsync(cols[o].nulls->Data(), 0, cols[o].nulls->Bytes(), s), "reset nulls");
        }
        CudaCheck(cudaMemsetAsync(cnt.Get(), 0, 4 * sizeof(unsigned long long), s), "reset counters");
        e.forcedOverflow = forced.Get();
        CudaCheck(omg::LaunchAggExtract(e, s), "extract groups");
        counters_[0] += 2;
        CudaCheck(cudaMemcpyAsync(hc, cnt.Get(), sizeof(hc), cudaMemcpyDeviceToHost, s), "read extract counters");
        im.stream.Sync();
    }
    if (hc[1] != 0) {
        throw OmniException("OPERATOR_RUNTIME_ERROR", "sum_aggregator overflow.", -5);
    }
    const int64_t rows = static_cast<int64_t>(hc[0]);
    if (!plan_.dictInputs.empty()) {
        DecodeStrings(cols, rows, s);
    }
    std::vector<omg::OutColumn> outCols = cols;
    if (!deviceOutput_) {
        outCols = omg::CopyColumnsToHost(cols, rows, s);
        im.stream.Sync();
        for (auto &c : outCols) {
            c.hasNull = false;  // host vectors: HasNull() scans the bitmap
        }
    }
    for (auto *b : omg::CarveBatches(outCols, rows, plan_.rowsPerBatch)) {
        outputs_.push_back(b);
    }
    counters_[5] = rows;
}

int32_t HashAggregationOperator::GetOutput(VectorBatch **outputVecBatch)
{
    *outputVecBatch = nullptr;
    if (!hasInputedData_) {
        return 0;
    }
    if (!extracted_) {
        extracted_ = true;
        Extract();
    }
    if (outputs_.empty()) {
        SetStatus(OMNI_STATUS_FINISHED);
        return 0;
    }
    *outputVecBatch = outputs_.front();
    outputs_.pop_front();
    if (outputs_.empty()) {
        SetStatus(OMNI_STATUS_FINISHED);
    }
    return 1;
}

}  // namespace op
}  // namespace omniruntime
