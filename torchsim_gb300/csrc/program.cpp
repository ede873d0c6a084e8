// Host-side compiler from the reference's packed event stream to pulse
// programs (sequences of Op micro-step templates).
//
// The event semantics are those of the reference's real-subspace kernels
// (src/torchsim/_epg_cpu.cpp:3055-3127): per event, relax over `duration`,
// then an optional pre-shift, then the RF (inversion or rotation) or, for an
// ADC with the RECORD bit, the record, then a post-shift, then a spoil or a
// shift-after. Events of zero duration add no relaxation (exp(0) = 1 and the
// recovery 1 - exp(0) = 0 are exact), so their steps are appended to the op
// before them whenever the template still has room in order.
#include <cstring>
#include <mutex>
#include <string>

#include "tsg_internal.h"

namespace tsg {

namespace {

enum Step { S_SHIFT, S_ROTATE, S_INVERT, S_RECORD, S_SPOIL };

// Slot order of the Op template.
constexpr int SLOT_RELAX = 0, SLOT_SHIFT1 = 1, SLOT_RF = 2, SLOT_SHIFT2 = 3, SLOT_SPOIL1 = 4,
              SLOT_RECORD = 5, SLOT_SHIFT3 = 6, SLOT_SPOIL2 = 7;

struct Builder {
    Op op{};
    OpSource src{-1, -1, -1};
    float2 ph{0.f, 0.f};  // phase of the op's pulse, of its receiver
    std::vector<float2>* phases = nullptr;  // collected when event phases are given
    int pos = -1;  // last slot used; -1 = no op open
    int n[3] = {0, 0, 0};

    void flush(std::vector<Op>& ops, std::vector<OpSource>& srcs) {
        if (pos < 0) return;
        op.code |= (uint32_t(n[0]) << OP_SHIFT1_SHIFT) | (uint32_t(n[1]) << OP_SHIFT2_SHIFT) |
                   (uint32_t(n[2]) << OP_SHIFT3_SHIFT);
        ops.push_back(op);
        srcs.push_back(src);
        if (phases) phases->push_back(ph);
        op = Op{};
        src = OpSource{-1, -1, -1};
        ph = float2{0.f, 0.f};
        pos = -1;
        n[0] = n[1] = n[2] = 0;
    }

    void open(std::vector<Op>& ops, std::vector<OpSource>& srcs) {
        flush(ops, srcs);
        pos = SLOT_RELAX;
    }

    // The slot a step can take at or after the current position, or -1.
    int fit(Step s) const {
        switch (s) {
            case S_SHIFT: {
                const int slots[3] = {SLOT_SHIFT1, SLOT_SHIFT2, SLOT_SHIFT3};
                for (int k = 0; k < 3; ++k) {
                    if (slots[k] > pos) return slots[k];
                    if (slots[k] == pos && n[k] < 3) return slots[k];
                }
                return -1;
            }
            case S_ROTATE:
            case S_INVERT:
                return pos < SLOT_RF ? SLOT_RF : -1;
            case S_RECORD:
                return pos < SLOT_RECORD ? SLOT_RECORD : -1;
            case S_SPOIL:
                if (pos <= SLOT_SPOIL1) return SLOT_SPOIL1;
                if (pos <= SLOT_SPOIL2) return SLOT_SPOIL2;
                return -1;
        }
        return -1;
    }

    void place(Step s, float flip, int32_t record, int32_t event, std::vector<Op>& ops,
               std::vector<OpSource>& srcs, float phase = 0.f) {
        int slot = pos < 0 ? -1 : fit(s);
        if (slot < 0) {
            open(ops, srcs);
            slot = fit(s);
        }
        switch (slot) {
            case SLOT_SHIFT1: n[0]++; break;
            case SLOT_SHIFT2: n[1]++; break;
            case SLOT_SHIFT3: n[2]++; break;
            case SLOT_RF:
                op.code |= uint32_t(s == S_ROTATE ? RF_ROTATE : RF_INVERT) << OP_RF_SHIFT;
                op.flip = s == S_ROTATE ? flip : 0.f;
                src.rf_event = event;
                if (s == S_ROTATE) ph.x = phase;
                break;
            case SLOT_RECORD:
                op.code |= OP_RECORD;
                op.record = record;
                src.rec_event = event;
                ph.y = phase;
                break;
            case SLOT_SPOIL1: op.code |= OP_SPOIL1; break;
            case SLOT_SPOIL2: op.code |= OP_SPOIL2; break;
            default: break;
        }
        pos = slot;
    }
};

}  // namespace

int compile_program(const float* duration, const int32_t* kind, const float* flip,
                    const uint8_t* action, const int32_t* output_index, int64_t trains,
                    int64_t events, bool unmerged, const float* duration_tangent,
                    HostProgram* out, const float* phase) {
    if (trains < 1 || events < 0)
        return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (events > 0 && (!duration || !kind || !flip || !action || !output_index))
        return fail(TSG_ERR_ARGUMENT, "null event buffer");
    if (events > (int64_t(1) << 30))
        return fail(TSG_ERR_CAPACITY, "event stream longer than 2^30 events");
    int32_t outputs = 0;
    for (int64_t e = 0; e < events; ++e) {
        if (kind[e] == 2 && (action[e] & A_RECORD)) {
            if (output_index[e] < 0)
                return fail(TSG_ERR_ARGUMENT, "recorded ADC event without an output index");
            outputs = std::max(outputs, output_index[e] + 1);
        }
    }
    std::vector<std::vector<Op>> per_train(trains);
    std::vector<std::vector<OpSource>> per_src(trains);
    std::vector<std::vector<float2>> per_phase(phase ? trains : 0);
    bool sequential = true;
    for (int64_t t = 0; t < trains; ++t) {
        auto& ops = per_train[t];
        auto& srcs = per_src[t];
        Builder b;
        if (phase) b.phases = &per_phase[t];
        int32_t expected = 0;
        for (int64_t e = 0; e < events; ++e) {
            const int64_t te = t * events + e;
            const float dt = duration[te];
            const float ddt = duration_tangent ? duration_tangent[te] : 0.f;
            const uint8_t a = action[e];
            if (unmerged || dt != 0.f || ddt != 0.f) {
                b.open(ops, srcs);
                b.op.code |= OP_RELAX;
                b.op.dt = dt;
                b.src.dt_event = int32_t(e);
            }
            if (a & A_PRE_SHIFT) b.place(S_SHIFT, 0.f, 0, int32_t(e), ops, srcs);
            const float pe = phase ? phase[te] : 0.f;
            if (kind[e] == 1) {
                if (a & A_INVERSION)
                    b.place(S_INVERT, 0.f, 0, int32_t(e), ops, srcs);
                else
                    b.place(S_ROTATE, flip[te], 0, int32_t(e), ops, srcs, pe);
            } else if (kind[e] == 2 && (a & A_RECORD)) {
                if (output_index[e] != expected) sequential = false;
                expected = output_index[e] + 1;
                b.place(S_RECORD, 0.f, output_index[e], int32_t(e), ops, srcs, pe);
            }
            if (a & A_POST_SHIFT) b.place(S_SHIFT, 0.f, 0, int32_t(e), ops, srcs);
            if (a & A_SPOIL_AFTER)
                b.place(S_SPOIL, 0.f, 0, int32_t(e), ops, srcs);
            else if (a & A_SHIFT_AFTER)
                b.place(S_SHIFT, 0.f, 0, int32_t(e), ops, srcs);
        }
        b.flush(ops, srcs);
    }
    size_t longest = 0;
    for (auto& v : per_train) longest = std::max(longest, v.size());
    if (longest > size_t(1) << 30) return fail(TSG_ERR_CAPACITY, "program too long");
    out->trains = trains;
    out->events = events;
    out->ops = int64_t(longest);
    out->outputs = outputs;
    out->sequential_records = sequential;
    out->op.assign(size_t(trains) * longest, Op{});
    out->src.assign(size_t(trains) * longest, OpSource{-1, -1, -1});
    for (int64_t t = 0; t < trains; ++t) {
        std::copy(per_train[t].begin(), per_train[t].end(), out->op.begin() + t * longest);
        std::copy(per_src[t].begin(), per_src[t].end(), out->src.begin() + t * longest);
    }
    out->phase.clear();
    if (phase) {
        out->phase.assign(size_t(trains) * longest, float2{0.f, 0.f});
        for (int64_t t = 0; t < trains; ++t)
            std::copy(per_phase[t].begin(), per_phase[t].end(), out->phase.begin() + t * longest);
    }
    return TSG_OK;
}

// ---- error reporting -------------------------------------------------------

namespace {
thread_local std::string g_last_error;
}

int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}

int cuda_fail(cudaError_t err, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(err);
    return TSG_ERR_CUDA;
}

}  // namespace tsg

extern "C" const char* tsg_last_error(void) { return tsg::g_last_error.c_str(); }
