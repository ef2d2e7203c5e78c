// nc_dense.cu — the dense form of the NeuCor step: a synapse pass and a neuron pass.
//
// The event form (nc_kernels.cu) pushes every launched spike from its source into the
// target's CSC row: scattered term writes and ring atomics per synaptic event.  When a
// large share of neurons fires every step (the kNN / U[0,1]-weight networks saturate
// near one fire per refractory period), nearly every in-row is touched every step
// anyway, and streaming the rows in order is cheaper than scattering into them.
//
//   k_dense_synapses (warp per span of 8 x 32 in-synapses, CSC order; the span's
//   streams arrive by bulk copies into shared memory, the next ones in flight while a
//   warp works), for the step prev = t-1 of the span's net:
//     Synapse::fire of every in-synapse whose source fired at prev (src/NeuCor.cpp:
//     727-738): dropped while busy, otherwise it captures fl(fl(0.2f*52)*w) and its
//     arrival step; then the plasticity of prev (src/NeuCor.cpp:740-761): post-spike
//     branch on the rows of targets that fired at prev, arrival branch on synapses
//     whose spike arrived at prev.  Launched terms are computed 32 at a time from a
//     per-warp queue so the two FP64 multiplies run on full warps.  Each chunk's
//     ballot of "arrived in t-KC .. t-1" is one word of the window bitmap.
//   k_dense_neurons (lane per neuron): charge_insynapses in ascending source order
//     from the window bitmap, charge_passive, threshold, AP, background draws (as the
//     event form's k_neuron_step); a neuron inside its AP skips its fold.  It also
//     writes each neuron's post state for the next synapse pass.
//   k_dense_fused: both passes of several steps in one cooperative launch, with grid
//     barriers between them (batched engines).
//
// Launches of the fires of prev happen at the start of step t instead of the end of
// step prev; nothing between those points reads what they write (a spike launched at
// prev arrives at prev+1 at the earliest and joins the fold from prev+2), so the
// results are the event form's bit for bit.  The launch decision reads the same rule:
// accepted iff prev - last_arrival >= KC + [target caller id > source caller id], and
// the captured weight includes the target's post-spike plasticity of prev when the
// target fired at prev and its caller id is below the source's.  A flush (before
// read-back) runs the synapse pass early; the step then finds it done (stdp_done) and
// its window bitmap already written.
#include "nc_device.cuh"
#include "nc_engine.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

namespace {

using namespace nc_dev;

constexpr int kMaxWarps = 8;  // 256 threads per block at most
constexpr int kQueue = 64;    // launched-term queue per warp

// Programmatic dependent launch: each pass of the dense step is launched so that its
// blocks may be scheduled while the previous pass drains, and waits here, before it
// reads anything, until that pass has completed and its writes are visible.  (A kernel
// launched without the attribute passes the wait at once.)
#ifndef NC_PDL
#define NC_PDL 1
#endif
__device__ __forceinline__ void wait_previous_pass()
{
    if (NC_PDL) asm volatile("griddepcontrol.wait;" ::: "memory");
}

// The synapse pass lets the neuron pass's blocks be scheduled once its own wait has
// passed (so the neuron pass that follows cannot start before the one that preceded has
// completed); the neuron pass then reads what no synapse pass writes (step counters, last
// fires, potentials, row bounds, input draws) before its own wait.
#ifndef NC_NEURON_EARLY_START
#define NC_NEURON_EARLY_START 1
#endif
__device__ __forceinline__ void release_next_pass()
{
    if (NC_PDL && NC_NEURON_EARLY_START) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Adds each warp's per-net counters (K of them, into stats[first ..]) to the nets'
// stats, summed per net over the block first.
template <int K>
__device__ void block_counters(const NcPools& P, int* s_net, unsigned long long (*s_acc)[2], int wib, int lane,
                               int acc_net, const unsigned long long* acc, int first)
{
    if (lane == 0) {
        s_net[wib] = acc_net;
#pragma unroll
        for (int k = 0; k < K; ++k) s_acc[wib][k] = acc[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int wpb = blockDim.x >> 5;
        for (int w = 0; w < wpb; ++w) {
            const int n = s_net[w];
            if (n < 0) continue;
            unsigned long long tot[K];
#pragma unroll
            for (int k = 0; k < K; ++k) tot[k] = s_acc[w][k];
            for (int v = w + 1; v < wpb; ++v) {
                if (s_net[v] != n) continue;
#pragma unroll
                for (int k = 0; k < K; ++k) tot[k] += s_acc[v][k];
                s_net[v] = -1;
            }
            unsigned long long* st = P.nets[n].stats;
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (tot[k]) atomicAdd(st + first + k, tot[k]);
        }
    }
}

// ---------------------------------------------------------------- staged synapse pass
// The same pass with the six in-synapse streams staged into shared memory by the
// bulk-copy (TMA) engine.  A warp works through its spans in units of half a span
// (4 chunks, 128 synapses) and keeps the next unit's copies in flight while it works
// on the current one (a ring of stage buffers, one mbarrier each): the memory system
// sees the copies in flight whatever the warp's registers hold, and 24 warps per SM
// (8 per block, 3 blocks) cover the compute's own latencies.  Shapes measured on the
// 100k x 100 network (us per pass, before the span-level values were shared by a
// span's units): 8 warps / half-span units / 2 stages 103, 6 / whole spans / 2 stages
// 104, 4 / whole / 2 105, 6 / half / 3 110, 4 / half / 4 119, 4 / whole / 3 136; after:
// a unit's four chunks gathered together 95.5 against two at a time 99.3, and 3 stages
// 104.8.

#ifndef NC_STAGE_WARPS
#define NC_STAGE_WARPS 8
#endif
#ifndef NC_STAGE_UNIT
#define NC_STAGE_UNIT 4
#endif
#ifndef NC_STAGE_DEPTH
#define NC_STAGE_DEPTH 2
#endif
constexpr int kStageWarps = NC_STAGE_WARPS;  // warps per block
constexpr int kUnitChunks = NC_STAGE_UNIT;   // chunks per staged unit
constexpr int kUnitSyn = kUnitChunks * 32;
constexpr int kUnitsPerSpan = NC_SPAN_CHUNKS / kUnitChunks;
constexpr int kStages = NC_STAGE_DEPTH;      // units in flight per warp, the current one included
#ifndef NC_STAGE_UNROLL
#define NC_STAGE_UNROLL 4
#endif
constexpr int kStageUnroll = NC_STAGE_UNROLL;  // chunks whose gathers are in flight together
static_assert(NC_SPAN_CHUNKS % kUnitChunks == 0 && kUnitChunks % kStageUnroll == 0, "unit shape");

struct StageBuf {                 // one unit, as laid out in the pools (16-byte multiples)
    int32_t pre[kUnitSyn];
    int32_t post[kUnitSyn];
    int32_t la[kUnitSyn];
    float w[kUnitSyn];
    int32_t ta[kUnitSyn];
    uint16_t dl[kUnitSyn];
};

struct NetConst {                 // a span's net constants (see the staged pass)
    const uint32_t* fprev;        // fired bits of prev
    const float* pst;             // per neuron: post trace at prev, -0.0 when it fired at prev
    const float* tab_pre;         // presynaptic trace table
    double e_term;
    int32_t t, kc, tab_pre_len;
    float dt, c52;
    Rates R;
};

// Lane 0's memo of the last span and net it staged: the second half of a span, and
// every span of a net after its first, are issued without reloading the span table
// and the net's descriptor (two dependent loads ahead of the copies).
// (Kept in the warp's shared memory: only lane 0 uses it.)
struct StageMemo {
    int64_t base;    // syn_base
    int64_t chunks;  // 32-synapse chunks of the net
    NcTile span;
    int sp;
    int net;
    int ok;          // the net runs its synapse pass in this launch
    int pad;
};

struct __align__(16) WarpStage {
    StageBuf buf[kStages];
    StageMemo memo;
    NetConst nc;
    unsigned long long bar[kStages];  // mbarriers: the copies of buf[k] have landed
    int32_t qs[kQueue];               // launched synapse, relative to its span's first
    float qx[kQueue];
};

constexpr size_t kStageSmem = sizeof(WarpStage) * kStageWarps;
constexpr uint32_t kWaitLimit = 1u << 22;  // try_wait polls before a stage gives up

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

#ifndef NC_STAGE_MEMO
#define NC_STAGE_MEMO 1
#endif

// Lane 0: copies unit `half` of span `sp` into b (all six streams), completing on *bar.
// Returns 0 when nothing is copied: the span's net is skipped this launch, or the unit
// lies past the net's last synapse.
__device__ int stage_unit(const NcPools& P, int sp, int half, bool flush, StageBuf* b, unsigned long long* bar,
                          StageMemo& m)
{
    if (!NC_STAGE_MEMO || sp != m.sp) {
        m.span = P.spans[sp];
        m.sp = sp;
    }
    if (!NC_STAGE_MEMO || m.span.net != m.net) {
        const NcNetDesc& D = P.nets[m.span.net];
        const int32_t t = D.t, prev = t - 1;
        m.ok = D.active && prev >= 1 && D.stdp_done < prev && (flush || t <= D.t_end);
        m.base = D.syn_base;
        m.chunks = (D.n_syn + 31) / 32;
        m.net = m.span.net;
    }
    if (!m.ok) return 0;
    const int64_t c0 = m.span.first + (int64_t)half * kUnitChunks;
    const int64_t nch = min((int64_t)kUnitChunks, m.chunks - c0);
    if (nch <= 0) return 0;
    const int64_t s = m.base + c0 * 32;
    const uint32_t b4 = (uint32_t)(nch * 128), b2 = (uint32_t)(nch * 64);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_addr(bar)), "r"(5 * b4 + b2)
                 : "memory");
    bulk_copy(b->pre, P.csc_pre + s, b4, bar);
    bulk_copy(b->post, P.csc_post + s, b4, bar);
    bulk_copy(b->la, P.la_c + s, b4, bar);
    bulk_copy(b->w, P.w + s, b4, bar);
    bulk_copy(b->ta, P.t_arr + s, b4, bar);
    bulk_copy(b->dl, P.csc_dl + s, b2, bar);
    return 1;
}

#ifndef NC_FULL_UNIT
#define NC_FULL_UNIT 1
#endif
template <bool B>
struct BoolTag {
    static constexpr bool value = B;
};

// All lanes: bounded wait for the phase of *bar.
__device__ __forceinline__ bool stage_wait(unsigned long long* bar, uint32_t phase)
{
    const uint32_t a = smem_addr(bar);
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(a), "r"(phase) : "memory");
        if (done) return true;
    }
    return false;
}

// The block's shared memory besides the stage buffers, used by both passes.
struct PassShared {
    int s_net[kMaxWarps];
    unsigned long long s_acc[kMaxWarps][2];
    int s_last;
    int s_ok;
    int s_cnt[kMaxWarps];
    uint16_t s_list[kMaxWarps * 32];
    float s_pot[kMaxWarps * 32];
};

// Lane 0 initialises the warp's stage barriers (once per launch).
__device__ __forceinline__ void init_stages(WarpStage& ws, int lane)
{
    if (lane == 0) {
        for (int k = 0; k < kStages; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&ws.bar[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
}

// The synapse pass of every span (see k_dense_synapses), each warp striding over the
// grid's spans.  phases: the parity of each stage slot's next completion, carried from
// one pass to the next within a launch.  All threads of the block call it.
template <bool kFlush>
__device__ __forceinline__ void synapse_pass(const NcPools& P, WarpStage& ws, PassShared& sh, uint32_t& phases)
{
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * kStageWarps + wib;
    const int nw = gridDim.x * kStageWarps;
    const int n_spans = P.n_spans_dev ? *P.n_spans_dev : P.n_spans;

    // unit k of this warp: half k % kUnitsPerSpan of span gw + (k / kUnitsPerSpan) * nw,
    // staged in slot k % kStages
    int iss = 0;  // lane 0: bit j set = slot j holds an issued unit not yet consumed
    StageMemo& memo = ws.memo;
    if (lane == 0) {
        memo.sp = -1;
        memo.net = -1;
    }
    if (lane == 0)
        for (int k = 0; k < kStages - 1; ++k) {
            const int sp = gw + (k / kUnitsPerSpan) * nw;
            if (sp < n_spans && stage_unit(P, sp, k % kUnitsPerSpan, kFlush, &ws.buf[k], &ws.bar[k], memo))
                iss |= 1 << k;
        }

    int acc_net = -1, cur_net = -1;
    unsigned long long acc[2] = {0, 0};  // launched, dropped
    bool ok = true;
    int qn = 0, nl = 0, nd = 0;
    for (int i = 0;; ++i) {
        const int sp = gw + i * nw;
        if (sp >= n_spans) break;
        // the span's values, once for its units
        const NcTile span = P.spans[sp];
        const NcNetDesc& D = P.nets[span.net];
        const int32_t t = D.t;
        const int32_t prev = t - 1;
        if (span.net != acc_net) {
            if (acc_net >= 0 && lane == 0) {
                unsigned long long* st = P.nets[acc_net].stats;
                atomicAdd(st + 1, acc[0]);
                atomicAdd(st + 2, acc[1]);
            }
            acc_net = span.net;
            acc[0] = acc[1] = 0;
        }
        const int64_t sb = D.syn_base;
        const int64_t nsyn = D.n_syn;
        const int64_t s_span = sb + (int64_t)span.first * 32;
        if (span.net != cur_net) {
            // the net's constants, once per warp in shared memory: reading them there needs
            // no reload after each global store (which could alias the descriptor) and no
            // registers across the chunk loop
            if (lane == 0) {
                NetConst& c = ws.nc;
                c.fprev = P.fired + (int64_t)(prev & 1) * P.total_words + D.word_base;
                c.pst = P.pst + D.neuron_base;
                c.tab_pre = P.tables + D.table_base;
                c.e_term = D.e_term;
                c.t = t;
                c.kc = D.kc;
                c.tab_pre_len = D.tab_pre_len;
                c.dt = D.dt;
                c.c52 = D.c52;
                c.R = rates_of(D);
            }
            __syncwarp();
            cur_net = span.net;
        }
        const NetConst& C = ws.nc;
#pragma unroll 1
        for (int half = 0; half < kUnitsPerSpan; ++half) {
            const int k = i * kUnitsPerSpan + half;
            const int slot = k % kStages;
            {
                // the slot consumed last iteration takes unit k + kStages - 1
                const int kn = k + kStages - 1, sn = kn % kStages;
                const int spn = gw + (kn / kUnitsPerSpan) * nw;
                if (lane == 0) {
                    iss &= ~(1 << sn);
                    if (spn < n_spans &&
                        stage_unit(P, spn, kn % kUnitsPerSpan, kFlush, &ws.buf[sn], &ws.bar[sn], memo))
                        iss |= 1 << sn;
                }
            }
            const int bits = __shfl_sync(kFull, iss, 0);
            if ((bits >> slot) & 1) {
                if (!stage_wait(&ws.bar[slot], (phases >> slot) & 1u)) {
                    if (lane == 0) atomicOr(P.dev_err, NC_DEV_ERR_STAGE_TIMEOUT);
                    ok = false;
                    break;
                }
                phases ^= 1u << slot;
                const StageBuf& B = ws.buf[slot];
                // this unit's synapses start at ubase; offsets within it are 32-bit
                const int64_t c0 = span.first + (int64_t)half * kUnitChunks;
                const int64_t ubase = sb + c0 * 32;
                const int32_t u_rem = (int32_t)min((int64_t)kUnitSyn, nsyn - c0 * 32);  // synapses in the unit
                int32_t* la_u = P.la_c + ubase;
                float* w_u = P.w + ubase;
                int32_t* ta_u = P.t_arr + ubase;
                uint32_t* win_u = P.win + (ubase >> 5);
                const uint32_t* inh_u = P.inh + (ubase >> 5);
                const int32_t qoff = half * kUnitSyn;  // the unit's first synapse, relative to the span
                const int32_t prev_c = C.t - 1;
                // the chunks of the unit; a full unit (all but a net's last) is compiled
                // without the per-lane bounds tests
                auto chunks = [&](auto all_tag) {
                constexpr bool kAll = decltype(all_tag)::value;
                for (int h = 0; h < kUnitChunks; h += kStageUnroll) {
                    uint32_t fword[kStageUnroll], ihw[kStageUnroll];
                    float pstv[kStageUnroll];
    #pragma unroll
                    for (int u = 0; u < kStageUnroll; ++u) {
                        const int q = (h + u) * 32 + lane;
                        fword[u] = 0u;
                        pstv[u] = 0.0f;
                        ihw[u] = 0u;
                        if (kAll || q < u_rem) {
                            fword[u] = C.fprev[B.pre[q] >> 5];
                            pstv[u] = C.pst[B.post[q]];
                            ihw[u] = __ldg(inh_u + h + u);
                        }
                    }
    #pragma unroll
                    for (int u = 0; u < kStageUnroll; ++u) {
                        const int q = (h + u) * 32 + lane;
                        const bool in = kAll || q < u_rem;
                        const int32_t la = B.la[q];
                        int32_t lac = in ? la : NC_NEVER;
                        bool launch = false, srcf = false;
                        float x = 0.0f;
                        if (in) {
                            const uint32_t dl = B.dl[q];
                            // target fired at prev: the sign of its post state
                            const bool tf = __float_as_uint(pstv[u]) == 0x80000000u;
                            srcf = (fword[u] >> (B.pre[q] & 31)) & 1u;
                            const bool arrived = la == prev_c;
                            const int32_t after = (int32_t)((dl >> 14) & 1u);
                            // free: never launched (NC_NEVER is INT32_MIN, far below) or
                            // prev - la >= KC + after
                            launch = srcf && la + C.kc + after <= prev_c;
                            const bool ih = (ihw[u] >> lane) & 1u;
                            const float lo = ih ? -1.0f : 0.0f, hi = ih ? 0.0f : 1.0f;
                            const float w0 = B.w[q];
                            float w1 = w0;
                            if (tf) w1 = plasticity_b(w0, lo, hi, trace_at_u(C.tab_pre, C.tab_pre_len, prev_c, B.ta[q]),
                                                      0.0f, C.R);
                            if (launch) {
                                // target below the source in caller order and fired at prev:
                                // its update ran first, post-spike plasticity included
                                const float cap = (((dl >> 15) & 1u) && tf) ? w1 : w0;
                                // AP_depolFac = 0.2f; *= 52.0; *= weight  (src/NeuCor.cpp:729-731)
                                x = C.dt * (C.c52 * cap);
                                lac = prev_c + (int32_t)(dl & 0x3fffu);
                                la_u[q] = lac;
                            }
                            float w2 = w1;
                            if (arrived) {
                                // the target's post trace at prev (0 when it fired at prev)
                                w2 = plasticity_b(w1, lo, hi, 0.0f, fabsf(pstv[u]), C.R);
                                ta_u[q] = prev_c;
                            }
                            if (tf || arrived) w_u[q] = w2;
                        }
                        // arrived t-KC .. t-1: in the fold of step t (NC_NEVER and later
                        // arrivals wrap past KC)
                        const bool win = (uint32_t)prev_c - (uint32_t)lac < (uint32_t)C.kc;
                        const uint32_t wm = __ballot_sync(kFull, win);
                        if (lane == 0 && (kAll || (h + u) * 32 < u_rem)) win_u[h + u] = wm;
                        const uint32_t lm = __ballot_sync(kFull, launch);
                        // launched and dropped, counted once per warp
                        const int nlm = __popc(lm);
                        nl += nlm;
                        nd += __popc(__ballot_sync(kFull, srcf)) - nlm;
                        if (lm) {
                            if (launch) {
                                const int pos = qn + __popc(lm & ((1u << lane) - 1u));
                                ws.qs[pos] = qoff + q;
                                ws.qx[pos] = x;
                            }
                            qn += __popc(lm);
                            if (qn >= 32) {
                                __syncwarp();
                                P.term[s_span + ws.qs[lane]] = make_term(ws.qx[lane], C.e_term);
                                __syncwarp();
                                if (lane < qn - 32) {
                                    ws.qs[lane] = ws.qs[32 + lane];
                                    ws.qx[lane] = ws.qx[32 + lane];
                                }
                                __syncwarp();
                                qn -= 32;
                            }
                        }
                    }
                }
                };
                if (NC_FULL_UNIT && u_rem == kUnitSyn) chunks(BoolTag<true>{});
                else chunks(BoolTag<false>{});
                // the queue holds offsets into this span: drain it before the warp moves on
                // to another span (the span's next unit follows when it was issued)
                const bool more = half + 1 < kUnitsPerSpan && ((bits >> ((k + 1) % kStages)) & 1);
                if (!more) {
                    __syncwarp();
                    if (lane < qn) P.term[s_span + ws.qs[lane]] = make_term(ws.qx[lane], C.e_term);
                    qn = 0;
                    acc[0] += (unsigned long long)nl;
                    acc[1] += (unsigned long long)nd;
                    nl = nd = 0;
                }
            }
            // the slot is refilled next iteration: finish reading it first, and order those
            // reads before the copy engine's writes
            __syncwarp();
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        if (!ok) break;
    }
    if (!ok) {
        // let this warp's copies in flight land (bounded) before the block's shared
        // memory goes away: the one that timed out and the ones issued behind it
        const int bits = __shfl_sync(kFull, iss, 0);
        for (int j = 0; j < kStages; ++j)
            if ((bits >> j) & 1) stage_wait(&ws.bar[j], (phases >> j) & 1u);
    }
    block_counters<2>(P, sh.s_net, sh.s_acc, wib, lane, acc_net, acc, 1);
}

#ifndef NC_STAGE_MIN_BLOCKS
#define NC_STAGE_MIN_BLOCKS 4
#endif

template <bool kFlush>
__global__ void __launch_bounds__(32 * kStageWarps, NC_STAGE_MIN_BLOCKS) k_dense_synapses(NcPools P)
{
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    __shared__ PassShared sh;
    WarpStage& ws = reinterpret_cast<WarpStage*>(dyn_smem)[threadIdx.x >> 5];
    init_stages(ws, threadIdx.x & 31);
    wait_previous_pass();
    release_next_pass();
    uint32_t phases = 0u;  // bit j: parity of slot j's next completion
    synapse_pass<kFlush>(P, ws, sh, phases);
}

// charge_insynapses (src/NeuCor.cpp:688-700) of neuron j of net D: the terms of the
// spikes that arrived t-1 .. t-KC, in ascending source id, folded into pot.  The row's
// window bits are read 256 synapses (8 words) at a time and streamed in batches of 8
// across word boundaries, so that a warp's batch count is its busiest lane's, not a sum
// of per-word maxima.
//
// When no term of the net can be negative (nonneg_terms), the running sum only grows
// (each `float += double` rounds a larger value, and rounding keeps the order), and so
// does charge_passive's result.  Once that result crosses the threshold the neuron fires
// whatever the remaining terms are, and its potential is then replaced by the AP table
// (src/NeuCor.cpp:682-686, 706-714): the fold stops there and returns the partial sum,
// which leads the update to the same decision.
__device__ __forceinline__ float fold_row(const NcPools& P, const NcNetDesc& D, int32_t j, float pot)
{
    const int64_t s0 = P.in_ptr[D.ptr_base + j];
    const int64_t s1 = P.in_ptr[D.ptr_base + j + 1];
    if (s1 <= s0) return pot;
    const bool stop = NC_FOLD_EARLY_EXIT && D.nonneg_terms;
    const float leak = D.leak;
    double pd = (double)pot;
    const int64_t wa0 = s0 >> 5, wa1 = (s1 - 1) >> 5;
    for (int64_t wb = wa0; wb <= wa1; wb += 8) {
        unsigned long long m[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t wq = wb + 2 * q;
            uint32_t x = wq <= wa1 ? P.win[wq] : 0u;
            uint32_t y = wq + 1 <= wa1 ? P.win[wq + 1] : 0u;
            if (wq == wa0) x &= ~0u << (s0 & 31);
            if (wq == wa1 && (s1 & 31)) x &= (1u << (s1 & 31)) - 1u;
            if (wq + 1 == wa1 && (s1 & 31)) y &= (1u << (s1 & 31)) - 1u;
            m[q] = x | ((unsigned long long)y << 32);
        }
        const double* tp = P.term + wb * 32;
        unsigned long long m0 = m[0], m1 = m[1], m2 = m[2], m3 = m[3];
        int base = 0;
        while (m0 | m1 | m2 | m3) {
            int b[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                // on to the next pair when this one is spent (an empty pair costs a slot)
                if (m0 == 0ull) {
                    m0 = m1;
                    m1 = m2;
                    m2 = m3;
                    m3 = 0ull;
                    base += 64;
                }
                b[k] = m0 ? base + __ffsll((long long)m0) - 1 : -1;
                m0 &= m0 - 1ull;
            }
            double v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (b[k] >= 0) v[k] = tp[b[k]];
            pd = fold8(pd, v, b, tp);
            // pd holds a float value exactly
            if (stop && fires_at((float)pd, leak)) return (float)pd;
        }
    }
    return __double2float_rn(pd);
}

// Lane per neuron (warp per tile of 32, a block per group of tiles).  Inside its AP
// (t - lastFire < KC) a neuron's potential comes from the AP table whatever its sum is,
// and it cannot cross the threshold, so its fold is skipped.  The block's remaining
// folds are packed onto its first threads before they run: a warp's FP64 add costs the
// same however few lanes are active, and at saturation two neurons in three are in
// their AP.
#ifndef NC_DNEURON_MAXT
#define NC_DNEURON_MAXT 256
#endif
#ifndef NC_DNEURON_MINB
#define NC_DNEURON_MINB NC_NEURON_MIN_BLOCKS
#endif
// The neuron pass of every tile (see k_dense_neurons), each block striding over groups
// of tiles; the last block to finish advances the nets' step counters.  All threads of
// the block call it.
#ifndef NC_NEURON_EARLY
#define NC_NEURON_EARLY 1
#endif

#ifndef NC_FOLD_PACK
#define NC_FOLD_PACK 1
#endif

__device__ __forceinline__ void neuron_pass(const NcPools& P, PassShared& sh)
{
    int* s_net = sh.s_net;
    int* s_cnt = sh.s_cnt;
    uint16_t* s_list = sh.s_list;
    float* s_pot = sh.s_pot;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int n_tiles = P.n_tiles_dev ? *P.n_tiles_dev : P.n_tiles;

    int acc_net = -1;
    unsigned long long acc[1] = {0};  // fires
    for (int tb = blockIdx.x; tb * wpb < n_tiles; tb += gridDim.x) {
        // which of the block's neurons fold, packed in tile order
        const int tix = tb * wpb + wib;
        bool need = false;
        // NC_NEURON_EARLY: the input requests and the background draw of each lane, which
        // do not depend on its potential, are made before the block's folds, so the warps
        // that do not fold make them while the others fold
        bool early_req = false;
        uint32_t early_bg = ~0u;  // slot of the background target for t+1, or ~0u
        if (tix < n_tiles) {
            const NcTile tile = P.tiles[tix];
            const NcNetDesc& D = P.nets[tile.net];
            const int32_t t = D.t;
            const int32_t j = tile.first + lane;
            if (D.active && t <= D.t_end && j < D.n) {
                const int32_t lf = P.lf[D.neuron_base + j];
                need = !(lf != NC_NEVER && t - lf < D.kc) &&
                       P.in_ptr[D.ptr_base + j + 1] > P.in_ptr[D.ptr_base + j];
                // with no negative term, a neuron already over the threshold fires whatever
                // its sum (see fold_row)
                if (NC_FOLD_EARLY_EXIT && need && D.nonneg_terms && fires_at(P.pot[D.neuron_base + j], D.leak))
                    need = false;
                if (NC_NEURON_EARLY) {
                    const int32_t pj = D.neuron_base + j;
                    const int32_t cid = D.permuted ? P.orig_id[pj] : j;
                    if (D.n_groups) early_req = input_request(P, D, cid, t);
                    if (D.bg_period > 0) {
                        uint32_t o[4];
                        philox((uint32_t)cid, (uint32_t)t, NC_STREAM_BACKGROUND, 0u, D, o);
                        if (o[0] % (uint32_t)D.bg_period == 0u) {
                            uint32_t tgt = o[1] % (uint32_t)D.n;
                            if (D.permuted) tgt = (uint32_t)P.slot_of[D.neuron_base + tgt];
                            early_bg = tgt;
                        }
                    }
                }
            }
        }
        // everything above reads state no synapse pass writes; the folds and the update
        // below need the synapse pass of this step
        if (NC_NEURON_EARLY_START) wait_previous_pass();
        if (NC_FOLD_PACK) {
            const uint32_t need_m = __ballot_sync(kFull, need);
            if (lane == 0) s_cnt[wib] = __popc(need_m);
            __syncthreads();
            int base = 0, total = 0;
            for (int w = 0; w < wpb; ++w) {
                base += w < wib ? s_cnt[w] : 0;
                total += s_cnt[w];
            }
            if (need) s_list[base + __popc(need_m & ((1u << lane) - 1u))] = (uint16_t)(wib * 32 + lane);
            __syncthreads();
            for (int r = threadIdx.x; r < total; r += blockDim.x) {
                const int ent = s_list[r];
                const NcTile tile = P.tiles[tb * wpb + (ent >> 5)];
                const NcNetDesc& D = P.nets[tile.net];
                const int32_t j = tile.first + (ent & 31);
                s_pot[ent] = fold_row(P, D, j, P.pot[D.neuron_base + j]);
            }
            __syncthreads();
        } else if (need) {
            // each lane folds its own neuron (no packing, no block barrier)
            const NcTile tile = P.tiles[tix];
            const NcNetDesc& D = P.nets[tile.net];
            const int32_t j = tile.first + lane;
            s_pot[wib * 32 + lane] = fold_row(P, D, j, P.pot[D.neuron_base + j]);
        }
        if (tix >= n_tiles) continue;
        const NcTile tile = P.tiles[tix];
        const NcNetDesc& D = P.nets[tile.net];
        const int32_t t = D.t;
        if (!(D.active && t <= D.t_end)) continue;
        if (tile.net != acc_net) {
            if (acc_net >= 0 && lane == 0) atomicAdd(P.nets[acc_net].stats + 0, acc[0]);
            acc_net = tile.net;
            acc[0] = 0;
        }
        const int32_t first = tile.first;
        const int32_t j = first + lane;
        const bool live = j < D.n;
        const int32_t pj = D.neuron_base + j;
        const int64_t word = D.word_base + (first >> 5);
        const int32_t kc = D.kc;
        bool fired = false;
        if (live) {
            int32_t lf = P.lf[pj];
            float pot = need ? s_pot[wib * 32 + lane] : P.pot[pj];
            const uint32_t fw = P.forced[(int64_t)(t & 1) * P.total_words + word];
            const uint32_t uw = P.ufire[(int64_t)(t & 1) * P.total_words + word];
            bool forced = (fw >> lane) & 1u;
            if (NC_NEURON_EARLY) forced = forced || early_req;
            else if (!forced && D.n_groups) forced = input_request(P, D, D.permuted ? P.orig_id[pj] : j, t);
            // charge_passive (src/NeuCor.cpp:677-680)
            pot = (pot - -70.0f) * D.leak + -70.0f;
            // charge_thresholdCheck (src/NeuCor.cpp:682-686); vesicles stay positive
            const bool can = (lf == NC_NEVER) || (t - lf >= kc);
            // an input firer's Neuron::fire has no threshold or refractory test
            fired = ((uw >> lane) & 1u) || ((-55.0f < pot || forced) && can);
            if (fired) {
                lf = t;
                P.lf[pj] = t;
                P.firings[pj] += 1u;
            }
            // AP (src/NeuCor.cpp:706-714)
            if (lf != NC_NEVER && t - lf < kc) pot = __ldg(P.tables + D.ap_base + (t - lf));
            P.pot[pj] = pot;
            // the post state the next synapse pass reads: getTrace at t (src/NeuCor.cpp:671-675,
            // 0 when it fired at t), its sign set when it fired at t
            P.pst[pj] = fired ? -0.0f : trace_at(P.tables + D.table_base + D.tab_pre_len, D.tab_post_len, t, lf);
        }
        const uint32_t fmask = __ballot_sync(kFull, fired);
        if (lane == 0) {
            P.fired[(int64_t)(t & 1) * P.total_words + word] = fmask;
            P.forced[(int64_t)(t & 1) * P.total_words + word] = 0u;
            P.ufire[(int64_t)(t & 1) * P.total_words + word] = 0u;
            if (D.raster_len > 0 && t >= D.raster_t0 && t - D.raster_t0 < D.raster_len)
                D.raster[(int64_t)(t - D.raster_t0) * D.n_words + (first >> 5)] = fmask;
        }
        acc[0] += (unsigned long long)__popc(fmask);
        // background fires for step t+1 (src/NeuCor.cpp:604-607), drawn per caller id
        if (NC_NEURON_EARLY && early_bg != ~0u)
            atomicOr(P.forced + (int64_t)((t + 1) & 1) * P.total_words + D.word_base + (early_bg >> 5),
                     1u << (early_bg & 31));
        if (!NC_NEURON_EARLY && live && D.bg_period > 0) {
            uint32_t o[4];
            philox((uint32_t)(D.permuted ? P.orig_id[pj] : j), (uint32_t)t, NC_STREAM_BACKGROUND, 0u, D, o);
            if (o[0] % (uint32_t)D.bg_period == 0u) {
                uint32_t tgt = o[1] % (uint32_t)D.n;
                if (D.permuted) tgt = (uint32_t)P.slot_of[D.neuron_base + tgt];
                atomicOr(P.forced + (int64_t)((t + 1) & 1) * P.total_words + D.word_base + (tgt >> 5),
                         1u << (tgt & 31));
            }
        }
    }
    // (a block with no tile of its own still waits before the step counters can move)
    if (NC_NEURON_EARLY_START) wait_previous_pass();
    block_counters<1>(P, s_net, sh.s_acc, wib, lane, acc_net, acc, 0);
    // the last block to finish advances the step counters
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) sh.s_last = (atomicAdd(P.done_ctr, 1u) == gridDim.x - 1u);
    __syncthreads();
    if (sh.s_last) {
        __threadfence();
        for (int n = threadIdx.x; n < P.n_nets; n += blockDim.x) {
            NcNetDesc* D = P.nets + n;
            if (D->active && D->t <= D->t_end) {
                if (D->stdp_done < D->t - 1) D->stdp_done = D->t - 1;
                D->stats[3] += 1ull;
                D->t += 1;
                D->tsum = __fadd_rn(D->tsum, D->dt);  // currentTime = targetTime (src/NeuCor.cpp:616)
            }
        }
        if (threadIdx.x == 0) *P.done_ctr = 0u;
    }
}

__global__ void __launch_bounds__(NC_DNEURON_MAXT, NC_DNEURON_MINB) k_dense_neurons(NcPools P)
{
    __shared__ PassShared sh;
    if (!NC_NEURON_EARLY_START) wait_previous_pass();
    neuron_pass(P, sh);
}

// ---------------------------------------------------------------- fused multi-step launch
// `ticks` whole steps of every net in one cooperative launch: synapse pass, grid
// barrier, neuron pass (whose last block advances the step counters), grid barrier.
// The grid is at most one wave (cudaLaunchCooperativeKernel refuses more), so every
// block reaches every barrier; each barrier wait is still bounded, and one that gives
// up sets NC_DEV_ERR_BARRIER and ends its block.  It saves the per-step launches and
// their drain and fill for batches of small networks.  (No periodic input firers: they
// run as their own kernel before a step.)
constexpr uint32_t kBarrierPolls = 1u << 24;  // polls (64 ns sleeps) before a barrier gives up

// bar[0]: arrivals, bar[1]: generation.  gen: this block's view of the generation.
__device__ bool grid_barrier(unsigned* bar, unsigned& gen, uint32_t* dev_err, PassShared& sh)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned g = gen;
        if (atomicAdd(&bar[0], 1u) == gridDim.x - 1u) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicExch(&bar[1], g + 1u);
        } else {
            uint32_t it = 0;
            while (atomicAdd(&bar[1], 0u) == g) {
                if (++it > kBarrierPolls) {
                    atomicOr(dev_err, NC_DEV_ERR_BARRIER);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        gen = g + 1u;
        sh.s_ok = ok;
    }
    __syncthreads();
    return sh.s_ok != 0;
}

#ifndef NC_FUSED_MIN_BLOCKS
#define NC_FUSED_MIN_BLOCKS 3  // the neuron pass needs ~80 registers
#endif
__global__ void __launch_bounds__(32 * kStageWarps, NC_FUSED_MIN_BLOCKS) k_dense_fused(NcPools P, int32_t ticks,
                                                                                     unsigned* bar)
{
    extern __shared__ __align__(128) unsigned char dyn_smem[];
    __shared__ PassShared sh;
    WarpStage& ws = reinterpret_cast<WarpStage*>(dyn_smem)[threadIdx.x >> 5];
    init_stages(ws, threadIdx.x & 31);
    unsigned gen = 0u;
    if (threadIdx.x == 0) gen = atomicAdd(&bar[1], 0u);
    uint32_t phases = 0u;
    for (int32_t k = 0; k < ticks; ++k) {
        synapse_pass<false>(P, ws, sh, phases);
        if (!grid_barrier(bar, gen, P.dev_err, sh)) return;
        neuron_pass(P, sh);
        if (!grid_barrier(bar, gen, P.dev_err, sh)) return;
        // the next pass's bulk copies read what other blocks stored in this launch
        asm volatile("fence.proxy.async.global;" ::: "memory");
    }
}

// After a flush: the synapse pass of every active net's last step is done.
__global__ void k_dense_mark_flushed(NcPools P)
{
    for (int n = threadIdx.x; n < P.n_nets; n += blockDim.x) {
        NcNetDesc* D = P.nets + n;
        if (D->active && D->stdp_done < D->t - 1) D->stdp_done = D->t - 1;
    }
}

// The synapse pass's grid: the launch configuration's, else a persistent grid of as
// many blocks as fit on the GPU at once (one wave; each warp strides over many spans,
// and keeps its next units' copies in flight meanwhile).  A grid of one span per warp
// measured 25% slower.  (A form of the pass on register loads instead of bulk copies
// measured 5% slower and was dropped.)
struct SynKernel {
    const void* fn;
    int threads;
    size_t smem;
};

template <bool kFlush>
SynKernel syn_kernel()
{
    return {(const void*)k_dense_synapses<kFlush>, 32 * kStageWarps, kStageSmem};
}

SynKernel fused_kernel() { return {(const void*)k_dense_fused, 32 * kStageWarps, kStageSmem}; }

// Blocks of one wave of kernel k on the current device (cached per device and kernel;
// the shared-memory opt-in is set here, before the first launch).  Returns 0 when the
// device cannot run it (the launch then reports an error).
int resident_blocks(const SynKernel& k, int which)
{
    static std::atomic<int> cache[3][64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int n = cache[which][dev].load(std::memory_order_relaxed);
    if (n == 0) {
        if (k.smem > 48 * 1024 &&
            cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem) != cudaSuccess)
            return 0;
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.threads, k.smem) != cudaSuccess ||
            sms * per_sm <= 0)
            return 0;
        n = sms * per_sm;
        cache[which][dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

template <bool kFlush>
int resident_syn_blocks()
{
    return resident_blocks(syn_kernel<kFlush>(), kFlush ? 1 : 0);
}

// Launches fn<<<grid, block, smem, s>>>(P) as a programmatic dependent launch.
cudaError_t launch_pdl(const void* fn, int grid, int block, size_t smem, cudaStream_t s, const NcPools& P)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = NC_PDL ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, (void (*)(NcPools))fn, P);
}

template <bool kFlush>
int launch_syn(const NcPools& P, const nc::LaunchShape& L, cudaStream_t s)
{
    const SynKernel k = syn_kernel<kFlush>();
    const int wpb = k.threads / 32;
    const int full = (P.n_spans + wpb - 1) / wpb;
    if (full <= 0) return 0;
    const int resident = resident_syn_blocks<kFlush>();
    if (resident <= 0) return -1;
    const int blocks = L.dense_blocks > 0 ? L.dense_blocks : (full < resident ? full : resident);
    return launch_pdl(k.fn, blocks, k.threads, k.smem, s, P) == cudaSuccess ? 0 : -1;
}

}  // namespace

namespace nc {

int launch_dense_synapses(const NcPools& P, const LaunchShape& L, void* stream)
{
    if (launch_syn<false>(P, L, (cudaStream_t)stream)) return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_dense_neurons(const NcPools& P, const LaunchShape& L, void* stream)
{
    const int wpb = L.neuron_block / 32;
    const int blocks = (P.n_tiles + wpb - 1) / wpb;
    if (blocks > 0 &&
        launch_pdl((const void*)k_dense_neurons, blocks, L.neuron_block, 0, (cudaStream_t)stream, P) != cudaSuccess)
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int prepare_dense_launch()
{
    return resident_syn_blocks<false>() > 0 && resident_syn_blocks<true>() > 0 &&
                   resident_blocks(fused_kernel(), 2) > 0
               ? 0
               : -1;
}

int launch_fused_dense(const NcPools& P, int32_t ticks, unsigned* bar, void* stream)
{
    if (ticks <= 0) return 0;
    const int resident = resident_blocks(fused_kernel(), 2);
    if (resident <= 0) return -1;
    // as many blocks as the larger pass has work for, at most one wave: a barrier over
    // fewer blocks is quicker
    const int need = std::max((P.n_spans + kStageWarps - 1) / kStageWarps, (P.n_tiles + kStageWarps - 1) / kStageWarps);
    const int blocks = std::max(1, std::min(resident, need));
    const cudaStream_t s = (cudaStream_t)stream;
    // the arrival count starts at zero (a barrier that gave up may have left it set)
    if (cudaMemsetAsync(bar, 0, sizeof(unsigned), s) != cudaSuccess) return -1;
    NcPools p = P;
    void* args[] = {(void*)&p, (void*)&ticks, (void*)&bar};
    if (cudaLaunchCooperativeKernel((const void*)k_dense_fused, dim3((unsigned)blocks), dim3(32 * kStageWarps),
                                    args, kStageSmem, s) != cudaSuccess)
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_step_dense(const NcPools& P, const LaunchShape& L, void* stream)
{
    return launch_dense_synapses(P, L, stream) | launch_dense_neurons(P, L, stream);
}

int launch_flush_dense(const NcPools& P, const LaunchShape& L, void* stream)
{
    if (launch_syn<true>(P, L, (cudaStream_t)stream)) return -1;
    k_dense_mark_flushed<<<1, 256, 0, (cudaStream_t)stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace nc
