// nc_kernels.cu — the NeuCor step on sm_103a.
//
// One simulation step t of every packed net is two launches:
//
//   k_neuron_step  (one warp per 32 neurons of one net)
//     a. plasticity deferred from step t-1 (src/NeuCor.cpp:740-761):
//        post-spike branch for every neuron that fired at t-1 (its whole in-synapse
//        row, the warp's 32 lanes striding it — coalesced), then the arrival branch
//        for every spike that arrived at t-1 (Synapse::run, src/NeuCor.cpp:718-726)
//     b. Neuron::run at t (src/NeuCor.cpp:619-641): charge_insynapses folds the
//        terms of spikes that arrived at t-1..t-KC in ascending source order (the
//        ring bits are in CSC order, so the fold follows std::map order), charge_passive,
//        charge_thresholdCheck with the forced-fire requests, AP
//     c. background fire draws for t+1 (src/NeuCor.cpp:604-607)
//     d. block-level compaction of the fired neurons into the fired list
//
//   k_spike_launch (one warp per fired neuron)
//     Synapse::fire (src/NeuCor.cpp:727-738) on each out-synapse: drop if busy,
//     capture fl(fl(0.2f*52)*w), compute the contribution term, mark the ring bit of
//     the arrival step.  The last block advances every net's step counter.
//
// The CPU restatement runs neurons in ascending id, each update firing at once.
// Two rules make the split launches produce the same bits:
//   * a synapse freed by its target's update at t (src/NeuCor.cpp:697) is free for
//     a launch at t only when the target's id is not above the source's
//     (free iff t - last_arrival >= KC + [target > source]);
//   * when the target also fired at t and precedes the source, the captured weight
//     includes the target's post-spike plasticity of t, computed on the fly.
// Plasticity of step t is written by the next k_neuron_step (or k_stdp_flush), so
// every launch at t reads weights as of the end of t-1.
//
// Floating point: built with --fmad=false so every multiply and add rounds on its
// own, as in the reference's x86-64 build.  The reference's transcendentals
// (powf, exp) are host-built tables indexed by step differences.
#include "nc_engine.cuh"

#include <cuda_runtime.h>

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float trace_at(const float* tab, int len, int32_t now, int32_t then)
{
    if (then == NC_NEVER) return 0.0f;  // lastSpikeArrival = -inf / lastFire = NaN
    const int32_t k = now - then;
    return k < len ? __ldg(tab + k) : 0.0f;
}

__device__ __forceinline__ bool inh_bit(const NcPools& P, int64_t s)
{
    return (__ldg(P.inh + (s >> 5)) >> (s & 31)) & 1u;
}

// The 32 inhibitory bits of synapses s .. s+31 (s need not be word-aligned; the pool
// keeps one spare word at its end).
__device__ __forceinline__ uint32_t inh_bits32(const NcPools& P, int64_t s)
{
    const int64_t w0 = s >> 5;
    return __funnelshift_r(__ldg(P.inh + w0), __ldg(P.inh + w0 + 1), (uint32_t)(s & 31));
}

// Synapse::synapticPlasticity weight update and clamp (src/NeuCor.cpp:757-761);
// fmin/fmax keep the C library's generic semantics.
__device__ __forceinline__ float plasticity(float w, bool inh, float traceS, float traceT, const NcNetDesc& D)
{
    const float weightChange = D.pre_factor * traceS - D.post_factor * traceT;
    float v = w + weightChange * D.lr;
    if (!inh) {
        const float m = (v <= 1.0f) ? v : 1.0f;
        v = (m >= 0.0f) ? m : 0.0f;
    } else {
        const float m = (v <= 0.0f) ? v : 0.0f;
        v = (m >= -1.0f) ? m : -1.0f;
    }
    return v;
}

// RN32 of a double, returned as the (exactly representable) double: the 52-bit
// fraction is rounded to 23 bits, half to even, with integer operations.  Values
// below the float normal range take the hardware conversion.  Together with one
// double add this is `float += double` (src/NeuCor.cpp:695) with one FP64 operation.
__device__ __forceinline__ double round_to_float(double d)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
    if (e < 1023u - 126u) return (double)__double2float_rn(d);
    u += 0x0FFFFFFFull + ((u >> 29) & 1ull);
    u &= ~0x1FFFFFFFull;
    return __longlong_as_double((long long)u);
}

__device__ __forceinline__ void philox(uint32_t a, uint32_t b, uint32_t stream, uint32_t c, const NcNetDesc& D,
                                       uint32_t out[4])
{
    nc_philox(a, b, stream, c, D.key0, D.key1, out);
}

// Whether input neuron j requests a fire at step t (Poisson groups).
__device__ bool input_request(const NcPools& P, const NcNetDesc& D, int32_t j, int32_t t)
{
    uint32_t o[4];
    for (int g = 0; g < D.n_groups; ++g) {
        const NcGroupDev G = P.groups[D.group_base + g];
        if (j < G.first || j >= G.first + G.count) continue;
        const uint32_t m = (uint32_t)(j - G.first);
        if (!G.correlated) {
            philox((uint32_t)G.index, (uint32_t)t, NC_STREAM_INDEPENDENT, m, D, o);
            if (o[0] < G.thresh) return true;
            continue;
        }
        for (int32_t src = t - G.jitter; src <= t + G.jitter; ++src) {
            if (src < 0) continue;
            philox((uint32_t)G.index, (uint32_t)src, NC_STREAM_SOURCE, 0u, D, o);
            if (!(o[0] < G.thresh)) continue;
            philox((uint32_t)G.index, (uint32_t)src, NC_STREAM_JITTER, m, D, o);
            const int32_t off = (int32_t)(o[0] % (uint32_t)(2 * G.jitter + 1)) - G.jitter;
            if (src + off == t) return true;
        }
    }
    return false;
}

// Pops up to 8 set bits of *m in ascending order into b[] (-1 when exhausted).
__device__ __forceinline__ void pop8(uint32_t* m, int b[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        b[k] = *m ? __ffs(*m) - 1 : -1;
        *m &= *m - 1u;
    }
}

// Deferred plasticity of step `prev` for the 32 neurons of a tile (all lanes call).
__device__ void tile_plasticity(const NcPools& P, const NcNetDesc& D, int64_t word, int lane, bool live,
                                int64_t s0, int64_t s1, int32_t r0, int32_t r1, int32_t lf, int32_t prev)
{
    const float* tab_pre = P.tables + D.table_base;
    const float* tab_post = tab_pre + D.tab_pre_len;
    // post-spike branch: the whole in-row of each neuron that fired at prev, the warp
    // striding it four chunks at a time so the loads of a chunk group overlap
    uint32_t m = P.fired[(int64_t)(prev & 1) * P.total_words + word];
    while (m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        const int64_t a0 = __shfl_sync(kFull, s0, b);
        const int64_t a1 = __shfl_sync(kFull, s1, b);
        for (int64_t base = a0; base < a1; base += 128) {
            float wv[4];
            int32_t ta[4];
            bool ok[4], ih[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t s = base + lane + 32 * u;
                ok[u] = s < a1;
                if (ok[u]) {
                    wv[u] = P.w[s];
                    ta[u] = P.t_arr[s];
                    ih[u] = inh_bit(P, s);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!ok[u]) continue;
                const int64_t s = base + lane + 32 * u;
                P.w[s] = plasticity(wv[u], ih[u], trace_at(tab_pre, D.tab_pre_len, prev, ta[u]), 0.0f, D);
            }
        }
    }
    __syncwarp();
    // arrival branch: spikes that arrived at prev (lastSpikeArrival = now; traceS = 0)
    if (live && r1 > r0) {
        const uint32_t* slot = P.ring + D.ring_base + (int64_t)(prev & D.ring_mask) * D.ring_words;
        const float trT = trace_at(tab_post, D.tab_post_len, prev, lf);
        for (int32_t wi = r0; wi < r1; ++wi) {
            uint32_t bits = slot[wi];
            if (!bits) continue;
            const int64_t cs = s0 + (int64_t)(wi - r0) * 32;
            const uint32_t ih = inh_bits32(P, cs);
            while (bits) {
                int b[8];
                pop8(&bits, b);
                float wv[8];
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (b[k] >= 0) wv[k] = P.w[cs + b[k]];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    if (b[k] < 0) continue;
                    P.t_arr[cs + b[k]] = prev;
                    P.w[cs + b[k]] = plasticity(wv[k], (ih >> b[k]) & 1u, 0.0f, trT, D);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_neuron_step(NcPools P)
{
    __shared__ int s_cnt[32];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    const int tick = *P.tick;
    const int n_tiles = P.n_tiles_dev ? *P.n_tiles_dev : P.n_tiles;

    // blocks stride over the tile table (block-uniform loop: the compaction barriers
    // below are reached by every thread)
    for (int base = blockIdx.x * wpb; base < n_tiles; base += gridDim.x * wpb) {
    const int gw = base + wib;
    uint32_t fmask = 0;
    int net = 0, first = 0;
    if (gw < n_tiles) {
        const NcTile tile = P.tiles[gw];
        const NcNetDesc& D = P.nets[tile.net];
        const int32_t t = D.t;
        if (D.active && t <= D.t_end) {
            net = tile.net;
            first = tile.first;
            const int32_t j = first + lane;
            const bool live = j < D.n;
            const int32_t pj = D.neuron_base + j;
            const int32_t pb = D.ptr_base + j;
            const int64_t word = D.word_base + (first >> 5);
            int32_t lf = NC_NEVER;
            int64_t s0 = 0, s1 = 0;
            int32_t r0 = 0, r1 = 0;
            if (live) {
                lf = P.lf[pj];
                s0 = P.in_ptr[pb];
                s1 = P.in_ptr[pb + 1];
                r0 = P.ring_off[pb];
                r1 = P.ring_off[pb + 1];
            }
            const int32_t prev = t - 1;
            if (prev >= 1 && D.stdp_done < prev) tile_plasticity(P, D, word, lane, live, s0, s1, r0, r1, lf, prev);

            bool fired = false;
            if (live) {
                const uint32_t fw = P.forced[(int64_t)(t & 1) * P.total_words + word];
                bool forced = (fw >> lane) & 1u;
                if (!forced && D.n_groups) forced = input_request(P, D, D.permuted ? P.orig_id[pj] : j, t);
                // charge_insynapses (src/NeuCor.cpp:688-700): terms of spikes that arrived
                // t-1 .. t-KC, ascending source id; the accumulator stays a float value
                float pot = P.pot[pj];
                if (r1 > r0) {
                    uint32_t* ring = P.ring + D.ring_base;
                    const int32_t oldest = t - D.kc;
                    double pd = (double)pot;
                    for (int32_t wi = r0; wi < r1; ++wi) {
                        uint32_t bits = 0, last = 0;
                        for (int32_t k = 1; k <= D.kc; ++k) {
                            if (t - k < 1) break;
                            last = ring[(int64_t)((t - k) & D.ring_mask) * D.ring_words + wi];
                            bits |= last;
                        }
                        const double* tp = P.term + s0 + (int64_t)(wi - r0) * 32;
                        while (bits) {
                            int b[8];
                            pop8(&bits, b);
                            double v[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (b[k] >= 0) v[k] = tp[b[k]];
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (b[k] >= 0) pd = round_to_float(__dadd_rn(pd, v[k]));
                        }
                        // the spikes that arrived KC steps ago are released (AP_fireTime = 0)
                        if (oldest >= 1 && last) ring[(int64_t)(oldest & D.ring_mask) * D.ring_words + wi] = 0u;
                    }
                    pot = __double2float_rn(pd);
                }
                // charge_passive (src/NeuCor.cpp:677-680)
                pot = (pot - -70.0f) * D.leak + -70.0f;
                // charge_thresholdCheck (src/NeuCor.cpp:682-686); vesicles stay positive
                const bool can = (lf == NC_NEVER) || (t - lf >= D.kc);
                fired = (-55.0f < pot || forced) && can;
                if (fired) {
                    lf = t;
                    P.lf[pj] = t;
                    P.firings[pj] += 1u;
                }
                // AP (src/NeuCor.cpp:706-714)
                if (lf != NC_NEVER && t - lf < D.kc) pot = __ldg(P.tables + D.ap_base + (t - lf));
                P.pot[pj] = pot;
            }
            fmask = __ballot_sync(kFull, fired);
            if (lane == 0) {
                P.fired[(int64_t)(t & 1) * P.total_words + word] = fmask;
                P.forced[(int64_t)(t & 1) * P.total_words + word] = 0u;
                if (D.raster_len > 0 && t >= D.raster_t0 && t - D.raster_t0 < D.raster_len)
                    D.raster[(int64_t)(t - D.raster_t0) * D.n_words + (first >> 5)] = fmask;
            }
            // background fires for step t+1 (src/NeuCor.cpp:604-607), drawn per caller id
            if (live && D.bg_period > 0) {
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
    }
    // block-level compaction of fired neurons
    const int cnt = __popc(fmask);
    if (lane == 0) s_cnt[wib] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const int c = s_cnt[w];
            s_cnt[w] = tot;
            tot += c;
        }
        s_base = tot ? atomicAdd(P.fired_count + (tick & 1), tot) : 0;
    }
    __syncthreads();
    if ((fmask >> lane) & 1u) {
        const int rank = __popc(fmask & ((1u << lane) - 1u));
        P.fired_list[(int64_t)(tick & 1) * P.fired_cap + s_base + s_cnt[wib] + rank] = make_int2(net, first + lane);
    }
    __syncthreads();  // s_cnt and s_base are reused by the next tile group
    }
}

__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__global__ void __launch_bounds__(256) k_spike_launch(NcPools P)
{
    __shared__ int s_last;
    __shared__ int s_net[32];
    __shared__ unsigned long long s_acc[32][3];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int nwb = blockDim.x >> 5;
    const int gw = blockIdx.x * nwb + wib;
    const int nw = gridDim.x * nwb;
    const int tick = *P.tick;
    const int par = tick & 1;
    const int count = P.fired_count[par];

    int acc_net = -1;
    unsigned long long acc_fire = 0, acc_launch = 0, acc_drop = 0;
    for (int e = gw; e < count; e += nw) {
        const int2 ent = P.fired_list[(int64_t)par * P.fired_cap + e];
        const NcNetDesc& D = P.nets[ent.x];
        const int32_t i = ent.y;
        const int32_t t = D.t;
        if (ent.x != acc_net) {
            if (acc_net >= 0 && lane == 0) {
                unsigned long long* st = P.nets[acc_net].stats;
                atomicAdd(st + 0, acc_fire);
                atomicAdd(st + 1, acc_launch);
                atomicAdd(st + 2, acc_drop);
            }
            acc_net = ent.x;
            acc_fire = acc_launch = acc_drop = 0;
        }
        const int64_t k0 = P.out_ptr[D.ptr_base + i];
        const int64_t k1 = P.out_ptr[D.ptr_base + i + 1];
        const uint32_t* fired_t = P.fired + (int64_t)(t & 1) * P.total_words + D.word_base;
        const float* tab_pre = P.tables + D.table_base;
        uint32_t* ring = P.ring + D.ring_base;
        int nl = 0, nd = 0;
        // four out-synapses per lane in flight: table loads, then weight loads, then writes
        for (int64_t kb = k0; kb < k1; kb += 128) {
            int32_t la[4], cs[4];
            uint32_t dl[4];
            bool ok[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t k = kb + lane + 32 * u;
                ok[u] = k < k1;
                if (ok[u]) {
                    dl[u] = (uint16_t)P.out_delay[k];
                    la[u] = P.last_arr[k];
                    cs[u] = P.out_csc[k];
                }
            }
            float wv[4];
            bool acc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                // freed by the target's update at t only if the target's id is not above
                acc[u] = ok[u] && (la[u] == NC_NEVER || t - la[u] >= D.kc + (int32_t)((dl[u] >> 14) & 1u));
                if (acc[u]) wv[u] = P.w[D.syn_base + cs[u]];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!ok[u]) continue;
                if (!acc[u]) {
                    ++nd;
                    continue;
                }
                const int64_t k = kb + lane + 32 * u;
                const int64_t s = D.syn_base + cs[u];
                float w = wv[u];
                if ((dl[u] >> 15) & 1u) {  // target id below the source's: its update ran first
                    const int32_t j = P.out_post[k];
                    if ((fired_t[j >> 5] >> (j & 31)) & 1u)
                        w = plasticity(w, inh_bit(P, s), trace_at(tab_pre, D.tab_pre_len, t, P.t_arr[s]), 0.0f, D);
                }
                // AP_depolFac = 0.2f; *= 52.0; *= weight  (src/NeuCor.cpp:729-731)
                const float depol = D.c52 * w;
                // deltaT*AP_depolFac*0.9943*exp(0.3702*deltaT)  (src/NeuCor.cpp:695)
                P.term[s] = __dmul_rn(__dmul_rn((double)(D.dt * depol), 0.9943), D.e_term);
                const int32_t d = (int32_t)(dl[u] & 0x3fffu);
                P.last_arr[k] = t + d;
                const uint32_t pos = P.out_ringpos[k];
                atomicOr(ring + (int64_t)((t + d) & D.ring_mask) * D.ring_words + (pos >> 5), 1u << (pos & 31));
                ++nl;
            }
        }
        nl = warp_sum(nl);
        nd = warp_sum(nd);
        acc_fire += 1;
        acc_launch += (unsigned long long)nl;
        acc_drop += (unsigned long long)nd;
    }
    // per-block reduction of the counters, per net
    if (lane == 0) {
        s_net[wib] = acc_net;
        s_acc[wib][0] = acc_fire;
        s_acc[wib][1] = acc_launch;
        s_acc[wib][2] = acc_drop;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < nwb; ++w) {
            const int n = s_net[w];
            if (n < 0) continue;
            unsigned long long f = s_acc[w][0], l = s_acc[w][1], d = s_acc[w][2];
            for (int v = w + 1; v < nwb; ++v) {
                if (s_net[v] != n) continue;
                f += s_acc[v][0];
                l += s_acc[v][1];
                d += s_acc[v][2];
                s_net[v] = -1;
            }
            unsigned long long* st = P.nets[n].stats;
            atomicAdd(st + 0, f);
            atomicAdd(st + 1, l);
            atomicAdd(st + 2, d);
        }
    }
    // the last block to finish advances the step counters
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(P.done_ctr, 1u) == gridDim.x - 1u);
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int n = threadIdx.x; n < P.n_nets; n += blockDim.x) {
            NcNetDesc* D = P.nets + n;
            if (D->active && D->t <= D->t_end) {
                if (D->stdp_done < D->t - 1) D->stdp_done = D->t - 1;
                D->stats[3] += 1ull;
                D->t += 1;
            }
        }
        if (threadIdx.x == 0) {
            P.fired_count[(tick + 1) & 1] = 0;
            *P.tick = tick + 1;
            *P.done_ctr = 0u;
        }
    }
}

// Applies the plasticity deferred from the last simulated step (before read-back).
__global__ void __launch_bounds__(256) k_stdp_flush(NcPools P)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gw >= P.n_tiles) return;
    const NcTile tile = P.tiles[gw];
    const NcNetDesc& D = P.nets[tile.net];
    const int32_t prev = D.t - 1;
    if (!D.active || prev < 1 || D.stdp_done >= prev) return;
    const int32_t j = tile.first + lane;
    const bool live = j < D.n;
    const int32_t pb = D.ptr_base + j;
    int32_t lf = NC_NEVER;
    int64_t s0 = 0, s1 = 0;
    int32_t r0 = 0, r1 = 0;
    if (live) {
        lf = P.lf[D.neuron_base + j];
        s0 = P.in_ptr[pb];
        s1 = P.in_ptr[pb + 1];
        r0 = P.ring_off[pb];
        r1 = P.ring_off[pb + 1];
    }
    tile_plasticity(P, D, D.word_base + (tile.first >> 5), lane, live, s0, s1, r0, r1, lf, prev);
}

__global__ void k_mark_flushed(NcPools P)
{
    for (int n = threadIdx.x; n < P.n_nets; n += blockDim.x) {
        NcNetDesc* D = P.nets + n;
        if (D->active && D->stdp_done < D->t - 1) D->stdp_done = D->t - 1;
    }
}

// Background draws made at step 0 for step 1 (the first NeuCor::run, src/NeuCor.cpp:604-607).
__global__ void k_background_prologue(NcPools P, int net)
{
    const NcNetDesc& D = P.nets[net];
    const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;  // caller id
    if (j >= D.n || D.bg_period <= 0) return;
    uint32_t o[4];
    philox((uint32_t)j, 0u, NC_STREAM_BACKGROUND, 0u, D, o);
    if (o[0] % (uint32_t)D.bg_period == 0u) {
        uint32_t tgt = o[1] % (uint32_t)D.n;
        if (D.permuted) tgt = (uint32_t)P.slot_of[D.neuron_base + tgt];
        atomicOr(P.forced + (int64_t)(1 & 1) * P.total_words + D.word_base + (tgt >> 5), 1u << (tgt & 31));
    }
}

// Forced fire requests for the net's next step (Neuron::scheduleFire).
__global__ void k_force_bits(NcPools P, int net, const int32_t* ids, int count)
{
    const NcNetDesc& D = P.nets[net];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int32_t j = ids[k];
    atomicOr(P.forced + (int64_t)(D.t & 1) * P.total_words + D.word_base + (j >> 5), 1u << (j & 31));
}

// Raster rows from device-slot order to caller-id order: thread per output word.
__global__ void k_raster_to_ids(const uint32_t* in, uint32_t* out, const int32_t* slot_of, int32_t n, int32_t n_words,
                                int32_t rows)
{
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)rows * n_words) return;
    const int32_t r = (int32_t)(q / n_words), w = (int32_t)(q % n_words);
    const uint32_t* row = in + (int64_t)r * n_words;
    uint32_t v = 0;
    for (int b = 0; b < 32; ++b) {
        const int32_t i = w * 32 + b;
        if (i >= n) break;
        const int32_t s = __ldg(slot_of + i);
        v |= ((__ldg(row + (s >> 5)) >> (s & 31)) & 1u) << b;
    }
    out[q] = v;
}

}  // namespace

namespace nc {

int launch_raster_to_ids(const uint32_t* in, uint32_t* out, const int32_t* slot_of, int32_t n, int32_t n_words,
                         int32_t rows, void* stream)
{
    const int64_t total = (int64_t)rows * n_words;
    if (total <= 0) return 0;
    k_raster_to_ids<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(in, out, slot_of, n, n_words,
                                                                                       rows);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}


static int check_launch()
{
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_neuron_step(const NcPools& P, const LaunchShape& L, void* stream)
{
    const int warps_per_block = L.neuron_block / 32;
    const int blocks = (P.n_tiles + warps_per_block - 1) / warps_per_block;
    if (blocks == 0) return 0;
    k_neuron_step<<<blocks, L.neuron_block, 0, (cudaStream_t)stream>>>(P);
    return check_launch();
}

int launch_spike_launch(const NcPools& P, const LaunchShape& L, void* stream)
{
    k_spike_launch<<<L.launch_blocks, L.launch_block, 0, (cudaStream_t)stream>>>(P);
    return check_launch();
}

int launch_stdp_flush(const NcPools& P, const LaunchShape& L, void* stream)
{
    const int warps_per_block = L.neuron_block / 32;
    const int blocks = (P.n_tiles + warps_per_block - 1) / warps_per_block;
    if (blocks > 0) k_stdp_flush<<<blocks, L.neuron_block, 0, (cudaStream_t)stream>>>(P);
    k_mark_flushed<<<1, 256, 0, (cudaStream_t)stream>>>(P);
    return check_launch();
}

int launch_background_prologue(const NcPools& P, int net, int n_neurons, void* stream)
{
    const int blocks = (n_neurons + 255) / 256;
    if (blocks > 0) k_background_prologue<<<blocks, 256, 0, (cudaStream_t)stream>>>(P, net);
    return check_launch();
}

int launch_force_bits(const NcPools& P, int net, const int32_t* d_ids, int count, void* stream)
{
    if (count <= 0) return 0;
    k_force_bits<<<(count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(P, net, d_ids, count);
    return check_launch();
}

}  // namespace nc
