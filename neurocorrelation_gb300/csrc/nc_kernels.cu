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
#include "nc_device.cuh"

#include <cuda_runtime.h>

namespace {

using namespace nc_dev;

// Post-spike branch of the plasticity of step `prev` (src/NeuCor.cpp:650-655, 740-761):
// the whole in-row of every neuron of the tile that fired at prev.  The warp takes the
// rows two at a time, each lane four synapses of each, so eight loads per lane are in
// flight per pass (all lanes call).
__device__ void postfire_rows(const NcPools& P, const NcNetDesc& D, int64_t word, int lane, int64_t s0, int64_t s1,
                              int32_t prev)
{
    const float* tab_pre = P.tables + D.table_base;
    const int32_t tpl = D.tab_pre_len;
    const Rates R = rates_of(D);
    uint32_t m = P.fired[(int64_t)(prev & 1) * P.total_words + word];
    while (m) {
        const int ba = __ffs(m) - 1;
        m &= m - 1;
        const bool pair = m != 0;
        const int bb = pair ? __ffs(m) - 1 : ba;
        if (pair) m &= m - 1;
        const int64_t a0 = __shfl_sync(kFull, s0, ba), a1 = __shfl_sync(kFull, s1, ba);
        const int64_t c0 = __shfl_sync(kFull, s0, bb);
        const int64_t c1 = pair ? __shfl_sync(kFull, s1, bb) : c0;
        const int64_t len = (a1 - a0) > (c1 - c0) ? (a1 - a0) : (c1 - c0);
        for (int64_t off = 0; off < len; off += 128) {
            float wv[8];
            int32_t ta[8];
            bool ok[8], ih[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t s = (u < 4 ? a0 : c0) + off + lane + 32 * (u & 3);
                ok[u] = s < (u < 4 ? a1 : c1);
                if (ok[u]) {
                    wv[u] = P.w[s];
                    ta[u] = P.t_arr[s];
                    ih[u] = inh_bit(P, s);
                }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (!ok[u]) continue;
                const int64_t s = (u < 4 ? a0 : c0) + off + lane + 32 * (u & 3);
                P.w[s] = plasticity(wv[u], ih[u], trace_at(tab_pre, tpl, prev, ta[u]), 0.0f, R);
            }
        }
    }
    __syncwarp();
}

// Arrival branch of the plasticity of step `prev` (Synapse::run, src/NeuCor.cpp:718-726:
// lastSpikeArrival = now, so traceS = 0) for one lane's in-row; used when the
// plasticity is flushed outside the step.
__device__ void arrival_row(const NcPools& P, const NcNetDesc& D, int64_t s0, int32_t r0, int32_t r1, int32_t lf,
                            int32_t prev)
{
    const float* tab_post = P.tables + D.table_base + D.tab_pre_len;
    const uint32_t* slot = P.ring + D.ring_base + (int64_t)(prev & D.ring_mask) * D.ring_words;
    const float trT = trace_at(tab_post, D.tab_post_len, prev, lf);
    const Rates R = rates_of(D);
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
                P.w[cs + b[k]] = plasticity(wv[k], (ih >> b[k]) & 1u, 0.0f, trT, R);
            }
        }
    }
}

__global__ void __launch_bounds__(256, NC_NEURON_MIN_BLOCKS) k_neuron_step(NcPools P)
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
            float pot = 0.0f;
            uint32_t fw = 0, uw = 0;
            if (live) {
                lf = P.lf[pj];
                s0 = P.in_ptr[pb];
                s1 = P.in_ptr[pb + 1];
                r0 = P.ring_off[pb];
                r1 = P.ring_off[pb + 1];
                pot = P.pot[pj];
                fw = P.forced[(int64_t)(t & 1) * P.total_words + word];
                uw = P.ufire[(int64_t)(t & 1) * P.total_words + word];
            }
            const int32_t prev = t - 1;
            const bool stdp = prev >= 1 && D.stdp_done < prev;
            if (stdp) postfire_rows(P, D, word, lane, s0, s1, prev);

            bool fired = false;
            if (live) {
                bool forced = (fw >> lane) & 1u;
                if (!forced && D.n_groups) forced = input_request(P, D, D.permuted ? P.orig_id[pj] : j, t);
                // charge_insynapses (src/NeuCor.cpp:688-700): terms of spikes that arrived
                // t-1 .. t-KC, ascending source id.  The arrival branch of the deferred
                // plasticity rides along: the spikes that arrived at prev are the ring
                // bits of slot prev.  Inside its AP (t - lastFire < KC) a neuron's
                // potential comes from the AP table whatever the sum is, and it cannot
                // cross the threshold, so only its sum is skipped.
                const bool in_ap = lf != NC_NEVER && t - lf < D.kc;
                if (r1 > r0) {
                    double pd = (double)pot;
                    // the sum is not needed inside the AP, nor, when no term can be
                    // negative, once the neuron is certain to fire (fires_at)
                    const bool stop = NC_FOLD_EARLY_EXIT && D.nonneg_terms;
                    bool settled = in_ap || (stop && fires_at(pot, D.leak));
                    uint32_t* ring = P.ring + D.ring_base;
                    const int64_t rw = D.ring_words;
                    const int32_t kc = D.kc;
                    const int32_t oldest = t - kc;
                    const float trT = trace_at(P.tables + D.table_base + D.tab_pre_len, D.tab_post_len, prev, lf);
                    const Rates R = rates_of(D);
                    for (int32_t wi = r0; wi < r1; wi += 2) {
                        const bool two = wi + 1 < r1;
                        uint32_t lo = 0, hi = 0, alo = 0, ahi = 0, olo = 0, ohi = 0;
                        for (int32_t k = 1; k <= kc && t - k >= 1; ++k) {
                            const uint32_t* row = ring + (int64_t)((t - k) & D.ring_mask) * rw + wi;
                            const uint32_t x = row[0];
                            const uint32_t y = two ? row[1] : 0u;
                            lo |= x;
                            hi |= y;
                            if (k == 1) {
                                alo = x;
                                ahi = y;
                            }
                            olo = x;  // ends as the word of slot t-KC when t-KC >= 1
                            ohi = y;
                        }
                        unsigned long long bits = settled ? 0ull : (lo | ((unsigned long long)hi << 32));
                        const unsigned long long arr = stdp ? (alo | ((unsigned long long)ahi << 32)) : 0ull;
                        const int64_t sb = s0 + (int64_t)(wi - r0) * 32;
                        unsigned long long ih = 0ull;
                        if (arr) ih = inh_bits32(P, sb) | ((unsigned long long)(two ? inh_bits32(P, sb + 32) : 0u) << 32);
                        // arrival branch first (it touches w and t_arr only, the fold reads term)
                        unsigned long long am = arr;
                        while (am) {
                            int b[8];
                            pop8_64(&am, b);
                            float wv[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (b[k] >= 0) wv[k] = P.w[sb + b[k]];
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                if (b[k] < 0) continue;
                                P.t_arr[sb + b[k]] = prev;
                                P.w[sb + b[k]] = plasticity(wv[k], (ih >> b[k]) & 1ull, 0.0f, trT, R);
                            }
                        }
                        while (bits) {
                            int b[8];
                            pop8_64(&bits, b);
                            double v[8];
                            const double* tp = P.term + sb;
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (b[k] >= 0) v[k] = tp[b[k]];
                            pd = fold8(pd, v, b, tp);
                            if (stop && fires_at((float)pd, D.leak)) {
                                settled = true;
                                bits = 0ull;
                            }
                        }
                        // the spikes that arrived KC steps ago are released (AP_fireTime = 0)
                        if (oldest >= 1) {
                            uint32_t* orow = ring + (int64_t)(oldest & D.ring_mask) * rw + wi;
                            if (olo) orow[0] = 0u;
                            if (two && ohi) orow[1] = 0u;
                        }
                    }
                    pot = __double2float_rn(pd);
                }
                // charge_passive (src/NeuCor.cpp:677-680)
                pot = (pot - -70.0f) * D.leak + -70.0f;
                // charge_thresholdCheck (src/NeuCor.cpp:682-686); vesicles stay positive
                const bool can = (lf == NC_NEVER) || (t - lf >= D.kc);
                // an input firer's Neuron::fire has no threshold or refractory test
                fired = ((uw >> lane) & 1u) || ((-55.0f < pot || forced) && can);
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
                P.ufire[(int64_t)(t & 1) * P.total_words + word] = 0u;
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

__global__ void __launch_bounds__(256, NC_LAUNCH_MIN_BLOCKS) k_spike_launch(NcPools P)
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
        // the descriptor's fields in registers: it lives in global memory, where every
        // store below could alias it
        const int32_t kc = D.kc, tpl = D.tab_pre_len, ring_mask = D.ring_mask;
        const int64_t syn_base = D.syn_base, ring_words = D.ring_words;
        const float dt = D.dt, c52 = D.c52;
        const Rates R = rates_of(D);
        const double e_term = D.e_term;
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
                acc[u] = ok[u] && (la[u] == NC_NEVER || t - la[u] >= kc + (int32_t)((dl[u] >> 14) & 1u));
                if (acc[u]) wv[u] = P.w[syn_base + cs[u]];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (!ok[u]) continue;
                if (!acc[u]) {
                    ++nd;
                    continue;
                }
                const int64_t k = kb + lane + 32 * u;
                const int64_t s = syn_base + cs[u];
                float w = wv[u];
                if ((dl[u] >> 15) & 1u) {  // target id below the source's: its update ran first
                    const int32_t j = P.out_post[k];
                    if ((fired_t[j >> 5] >> (j & 31)) & 1u)
                        w = plasticity(w, inh_bit(P, s), trace_at(tab_pre, tpl, t, P.t_arr[s]), 0.0f, R);
                }
                // AP_depolFac = 0.2f; *= 52.0; *= weight  (src/NeuCor.cpp:729-731)
                const float depol = c52 * w;
                // deltaT*AP_depolFac*0.9943*exp(0.3702*deltaT)  (src/NeuCor.cpp:695)
                P.term[s] = make_term(dt * depol, e_term);
                const int32_t d = (int32_t)(dl[u] & 0x3fffu);
                P.last_arr[k] = t + d;
                const uint32_t pos = P.out_ringpos[k];
                atomicOr(ring + (int64_t)((t + d) & ring_mask) * ring_words + (pos >> 5), 1u << (pos & 31));
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
                D->tsum = __fadd_rn(D->tsum, D->dt);  // currentTime = targetTime (src/NeuCor.cpp:616)
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
    postfire_rows(P, D, D.word_base + (tile.first >> 5), lane, s0, s1, prev);
    if (live && r1 > r0) arrival_row(P, D, s0, r0, r1, lf, prev);
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
