// nc_build.cu — construction of kNN networks on the device (nc_create_knn).
//
// The same network as nc_build_knn + nc_create (host), bit for bit, built on the GPU:
//   1. positions from Philox (k_positions) and a uniform grid of cells: points are
//      bucketed by cell (counts on the device, one scan on the host, a fill kernel);
//   2. the k nearest neighbours of every point (k_knn, warp per point): grid shells of
//      growing Chebyshev radius r, stopping under the host builder's own rule (k
//      candidates whose k-th distance is below r*h, or the whole grid), then the k
//      smallest (distance, id) pairs — a radix select of the k-th distance over the
//      candidates and a bitonic sort of the chosen ones in shared memory;
//   3. the in-synapse rows (CSC): in-degrees on the device, the row starts on the host,
//      an atomic scatter of the edges into their target's row and a per-row bitonic
//      sort by source id (warp per row), then the dense form's streams: source and target
//      slots, weight, delay (coord3::getDist, rounded to whole steps) and the same-step
//      order flags.
// Storage order (Morton codes, an O(n log n) sort of the positions) and the constant
// tables stay on the host.  Capacities are bounded (candidates per point, ties, row
// length); past them the build reports it and the host builder takes over.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "nc_net.h"

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kKnnWarps = 4;          // warps per block of k_knn
constexpr int kCandCap = 16384;       // candidates per point (global scratch per warp)
constexpr int kMaxK = 512;            // neighbours per point
constexpr int kTieCap = 256;          // candidates at exactly the k-th distance
constexpr int kRowCap = 2048;         // in-synapses per row sorted in shared memory
constexpr int kRowWarps = 4;

// build failure flags
constexpr uint32_t kFlagCandidates = 1u, kFlagTies = 2u, kFlagRow = 4u, kFlagDelay = 8u;

__device__ __forceinline__ float dist3(const float* a, const float* b)
{
    // coord3::getDist (src/NeuCor.h:16-18), the host's float operations in order
    const float dx = __fsub_rn(a[0], b[0]), dy = __fsub_rn(a[1], b[1]), dz = __fsub_rn(a[2], b[2]);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

__device__ __forceinline__ int32_t cell_of(float v, float h, int32_t g)
{
    const int32_t c = __float2int_rz(__fdiv_rn(v, h));
    return min(g - 1, max(0, c));
}

__global__ void k_positions(int32_t n, uint32_t k0, uint32_t k1, float side, float h, int32_t g, float* xyz,
                            int32_t* cell, int32_t* count)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t o[4];
    nc_philox((uint32_t)i, 0u, nc::kStreamPosition, 0u, k0, k1, o);
    float p[3];
    for (int a = 0; a < 3; ++a) {
        p[a] = __fmul_rn(nc::unit24(o[a]), side);
        xyz[3 * (int64_t)i + a] = p[a];
    }
    const int32_t c = (cell_of(p[0], h, g) * g + cell_of(p[1], h, g)) * g + cell_of(p[2], h, g);
    cell[i] = c;
    atomicAdd(count + c, 1);
}

__global__ void k_fill_cells(int32_t n, const int32_t* cell, int32_t* cursor, int32_t* members)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    members[atomicAdd(cursor + cell[i], 1)] = i;
}

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int* total)
{
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    *total = __shfl_sync(kFull, x, 31);
    return x - v;
}

// Rank `rank` (1-based) smallest of the high words of keys[0..count): a radix select
// over 8-bit digits with a histogram in shared memory.
__device__ uint32_t select_high(const unsigned long long* keys, int count, int rank, uint32_t* hist, int lane)
{
    uint32_t prefix = 0u, pmask = 0u;
    int remaining = rank;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = lane; b < 256; b += 32) hist[b] = 0u;
        __syncwarp();
        for (int c = lane; c < count; c += 32) {
            const uint32_t hk = (uint32_t)(keys[c] >> 32);
            if ((hk & pmask) == prefix) atomicAdd(hist + ((hk >> shift) & 255u), 1u);
        }
        __syncwarp();
        int local = 0;
        for (int q = 0; q < 8; ++q) local += (int)hist[lane * 8 + q];
        int tot = 0;
        const int before = warp_excl_scan(local, lane, &tot);
        const bool mine = before < remaining && remaining <= before + local;
        const unsigned who = __ballot_sync(kFull, mine);
        const int src = __ffs(who) - 1;
        int digit = 0, below = 0;
        if (lane == src) {
            int acc = before;
            for (int q = 0; q < 8; ++q) {
                const int h = (int)hist[lane * 8 + q];
                if (acc + h >= remaining) {
                    digit = lane * 8 + q;
                    break;
                }
                acc += h;
            }
            below = acc;
        }
        digit = __shfl_sync(kFull, digit, src);
        below = __shfl_sync(kFull, below, src);
        prefix |= (uint32_t)digit << shift;
        pmask |= 0xffu << shift;
        remaining -= below;
        __syncwarp();
    }
    return prefix;
}

// Ascending bitonic sort of a[0..p) (p a power of two) by one warp.
template <class T>
__device__ void warp_bitonic(T* a, int p, int lane)
{
    for (int kb = 2; kb <= p; kb <<= 1)
        for (int jb = kb >> 1; jb > 0; jb >>= 1) {
            for (int i = lane; i < p; i += 32) {
                const int l = i ^ jb;
                if (l > i) {
                    const T x = a[i], y = a[l];
                    const bool up = (i & kb) == 0;
                    if ((x > y) == up) {
                        a[i] = y;
                        a[l] = x;
                    }
                }
            }
            __syncwarp();
        }
}

struct KnnShared {
    uint32_t hist[kKnnWarps][256];
    unsigned long long sel[kKnnWarps][kMaxK];
    int32_t ties[kKnnWarps][kTieCap];
    int nsel[kKnnWarps], nties[kKnnWarps];
};

__global__ void __launch_bounds__(32 * kKnnWarps) k_knn(int32_t n, int32_t k, float h, int32_t g, uint32_t k0,
                                                        uint32_t k1, const float* xyz, const int32_t* cstart,
                                                        const int32_t* members, unsigned long long* scratch,
                                                        int32_t* to, float* weight, uint32_t* flags)
{
    __shared__ KnnShared sh;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * kKnnWarps + wib;
    const int nw = gridDim.x * kKnnWarps;
    unsigned long long* cand = scratch + (int64_t)gw * kCandCap;
    uint32_t* hist = sh.hist[wib];
    for (int32_t i = gw; i < n; i += nw) {
        const float pi[3] = {xyz[3 * (int64_t)i], xyz[3 * (int64_t)i + 1], xyz[3 * (int64_t)i + 2]};
        const int32_t cx = cell_of(pi[0], h, g), cy = cell_of(pi[1], h, g), cz = cell_of(pi[2], h, g);
        int count = 0;
        uint32_t kth = 0u;
        bool overflow = false;
        for (int32_t r = 0;; ++r) {
            // the shell of cells at Chebyshev distance r, lanes over the cube's cells
            const int32_t w = 2 * r + 1;
            const int64_t cube = (int64_t)w * w * w;
            for (int64_t base = 0; base < cube; base += 32) {
                const int64_t idx = base + lane;
                int32_t c = -1;
                if (idx < cube) {
                    const int32_t x = cx - r + (int32_t)(idx / ((int64_t)w * w));
                    const int32_t y = cy - r + (int32_t)((idx / w) % w);
                    const int32_t z = cz - r + (int32_t)(idx % w);
                    const int32_t cheb = max(abs(x - cx), max(abs(y - cy), abs(z - cz)));
                    if (cheb == r && x >= 0 && x < g && y >= 0 && y < g && z >= 0 && z < g) c = (x * g + y) * g + z;
                }
                const int32_t b0 = c >= 0 ? cstart[c] : 0, b1 = c >= 0 ? cstart[c + 1] : 0;
                int tot = 0;
                const int off = warp_excl_scan(b1 - b0, lane, &tot);
                if (count + tot > kCandCap) {
                    overflow = true;
                    break;
                }
                int q = count + off;
                for (int32_t m = b0; m < b1; ++m) {
                    const int32_t j = members[m];
                    if (j == i) continue;
                    const float d = dist3(pi, xyz + 3 * (int64_t)j);
                    cand[q++] = ((unsigned long long)__float_as_uint(d) << 32) | (uint32_t)j;
                }
                // shell 0 is i's own cell, written by lane 0 without i itself: its range
                // ends one short
                count += tot - (r == 0 ? 1 : 0);
                __syncwarp();
            }
            if (overflow) break;
            const bool all = r >= g;
            if (count >= k) {
                kth = select_high(cand, count, k, hist, lane);
                if (all || __uint_as_float(kth) < __fmul_rn(__int2float_rn(r), h)) break;
            } else if (all) {
                break;
            }
        }
        if (overflow) {
            if (lane == 0) atomicOr(flags, kFlagCandidates);
            continue;
        }
        // the k smallest (distance, id): every candidate below the k-th distance, then the
        // smallest ids at exactly that distance
        if (lane == 0) {
            sh.nsel[wib] = 0;
            sh.nties[wib] = 0;
        }
        __syncwarp();
        for (int c = lane; c < count; c += 32) {
            const unsigned long long key = cand[c];
            const uint32_t hk = (uint32_t)(key >> 32);
            if (hk < kth) {
                sh.sel[wib][atomicAdd(&sh.nsel[wib], 1)] = key;
            } else if (hk == kth) {
                const int t = atomicAdd(&sh.nties[wib], 1);
                if (t < kTieCap) sh.ties[wib][t] = (int32_t)(uint32_t)key;
            }
        }
        __syncwarp();
        const int nsel = sh.nsel[wib], nties = sh.nties[wib];
        if (nties > kTieCap) {
            if (lane == 0) atomicOr(flags, kFlagTies);
            continue;
        }
        int tp = 1;
        while (tp < nties) tp <<= 1;
        for (int t = nties + lane; t < tp; t += 32) sh.ties[wib][t] = 0x7fffffff;
        __syncwarp();
        warp_bitonic(sh.ties[wib], tp, lane);
        const int need = k - nsel;
        for (int t = lane; t < need; t += 32)
            sh.sel[wib][nsel + t] = ((unsigned long long)kth << 32) | (uint32_t)sh.ties[wib][t];
        int sp = 1;
        while (sp < k) sp <<= 1;
        for (int t = k + lane; t < sp; t += 32) sh.sel[wib][t] = ~0ull;
        __syncwarp();
        warp_bitonic(sh.sel[wib], sp, lane);
        // nc_build_knn's output: neighbours in ascending (distance, id), Philox weights
        for (int m = lane; m < k; m += 32) {
            const int64_t q = (int64_t)i * k + m;
            to[q] = (int32_t)(uint32_t)sh.sel[wib][m];
            uint32_t o[4];
            nc_philox((uint32_t)i, (uint32_t)(m >> 2), nc::kStreamWeight, 0u, k0, k1, o);
            weight[q] = nc::unit24(o[m & 3]);
        }
        __syncwarp();
    }
}

__global__ void k_indegree(int64_t edges, const int32_t* to, const int32_t* slot_of, int32_t* deg)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= edges) return;
    atomicAdd(deg + slot_of[to[e]], 1);
}

__global__ void k_scatter_rows(int64_t edges, int32_t k, const int32_t* to, const int32_t* slot_of,
                               unsigned long long* cursor, unsigned long long* rows)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= edges) return;
    const int32_t from = (int32_t)(e / k);
    const unsigned long long pos = atomicAdd(cursor + slot_of[to[e]], 1ull);
    rows[pos] = ((unsigned long long)(uint32_t)from << 32) | (uint32_t)e;
}

// Warp per target row: sort by source id, then the dense form's in-synapse streams.
__global__ void __launch_bounds__(32 * kRowWarps) k_fill_rows(NcPools P, int32_t n, int32_t k, float dt,
                                                              const float* xyz, const int32_t* to,
                                                              const float* weight, const int32_t* slot_of,
                                                              const unsigned long long* rows, int64_t* input_to_csc,
                                                              uint32_t* flags)
{
    __shared__ unsigned long long sh[kRowWarps][kRowCap];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * kRowWarps + wib;
    const int nw = gridDim.x * kRowWarps;
    for (int32_t tj = gw; tj < n; tj += nw) {
        const int64_t s0 = P.in_ptr[tj], s1 = P.in_ptr[tj + 1];
        const int len = (int)(s1 - s0);
        if (len > kRowCap) {
            if (lane == 0) atomicOr(flags, kFlagRow);
            continue;
        }
        int p = 1;
        while (p < len) p <<= 1;
        for (int q = lane; q < p; q += 32) sh[wib][q] = q < len ? rows[s0 + q] : ~0ull;
        __syncwarp();
        warp_bitonic(sh[wib], p, lane);
        for (int q = lane; q < len; q += 32) {
            const unsigned long long key = sh[wib][q];
            const int32_t from = (int32_t)(key >> 32);
            const int64_t e = (int64_t)(uint32_t)key;
            const int32_t target = to[e];
            const int64_t c = s0 + q;
            // AP_fireTime = length * AP_speed in whole steps (nc::delay_steps)
            const float len_ = dist3(xyz + 3 * (int64_t)from, xyz + 3 * (int64_t)target);
            const float qd = floorf(__fadd_rn(__fdiv_rn(__fmul_rn(len_, 2.0f), dt), 0.5f));
            int32_t d = 1;
            if (qd >= 1.0f) d = (int32_t)qd;
            if (qd > 16383.0f) {
                atomicOr(flags, kFlagDelay);
                d = 1;
            }
            const uint32_t fl = (target > from ? 1u << 14 : 0u) | (target < from ? 1u << 15 : 0u);
            P.csc_pre[c] = slot_of[from];
            P.csc_post[c] = tj;
            P.csc_dl[c] = (uint16_t)((uint32_t)d | fl);
            P.w[c] = weight[e];
            P.t_arr[c] = NC_NEVER;
            P.la_c[c] = NC_NEVER;
            input_to_csc[e] = c;
        }
        __syncwarp();
    }
}

template <class T>
T* dalloc(size_t count, std::vector<void*>& own, cudaError_t& e)
{
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (p) own.push_back(p);
    return (T*)p;
}

struct Frees {
    std::vector<void*> v;
    ~Frees()
    {
        for (void* p : v) cudaFree(p);
    }
};

}  // namespace

namespace nc {

// Builds the kNN network into `net` (host description and device pools).  Returns
// NC_OK, NC_ERR_UNSUPPORTED when a capacity of the device build was exceeded (the
// caller then builds on the host), or another NC_ERR_* code with `err` set.
int build_knn_device(int32_t n, int32_t k, float density, uint64_t seed, const nc_params& p, nc_net* net,
                     std::string& err)
{
    if (n < 2 || k < 1 || k >= n || k > kMaxK || !(density > 0.0f)) {
        err = "device kNN build: need 2 <= n, 1 <= k < n, k <= 512, density > 0";
        return NC_ERR_UNSUPPORTED;
    }
    if (p.step_mode != NC_STEP_DENSE) {
        err = "device kNN build: the dense form only";
        return NC_ERR_UNSUPPORTED;
    }
    if ((int64_t)n * k >= (1ll << 31)) {
        err = "too many synapses in one network";
        return NC_ERR_INVALID;
    }
    const KnnGrid G = knn_grid(n, k, density);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const int64_t cells = (int64_t)G.g * G.g * G.g;
    const int64_t edges = (int64_t)n * k;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    Frees own;
    cudaError_t e = cudaSuccess;
    float* d_xyz = dalloc<float>(3 * (size_t)n, own.v, e);
    int32_t* d_cell = dalloc<int32_t>((size_t)n, own.v, e);
    int32_t* d_count = dalloc<int32_t>((size_t)cells + 1, own.v, e);
    int32_t* d_members = dalloc<int32_t>((size_t)n, own.v, e);
    int32_t* d_to = dalloc<int32_t>((size_t)edges, own.v, e);
    float* d_w = dalloc<float>((size_t)edges, own.v, e);
    uint32_t* d_flags = dalloc<uint32_t>(1, own.v, e);
    const int knn_blocks = std::max(1, sms * 8);
    unsigned long long* d_scratch = dalloc<unsigned long long>((size_t)knn_blocks * kKnnWarps * kCandCap, own.v, e);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (allocation)", e);
        return e == cudaErrorMemoryAllocation ? NC_ERR_NOMEM : NC_ERR_CUDA;
    }
    cudaMemset(d_count, 0, sizeof(int32_t) * ((size_t)cells + 1));
    cudaMemset(d_flags, 0, sizeof(uint32_t));
    k_positions<<<(n + 255) / 256, 256>>>(n, k0, k1, G.side, G.h, G.g, d_xyz, d_cell, d_count);
    // cell starts (host scan of the counts)
    std::vector<int32_t> cstart((size_t)cells + 1, 0);
    e = cudaMemcpy(cstart.data() + 1, d_count, sizeof(int32_t) * (size_t)cells, cudaMemcpyDeviceToHost);
    for (int64_t c = 0; c < cells; ++c) cstart[(size_t)c + 1] += cstart[(size_t)c];
    if (e == cudaSuccess) e = cudaMemcpy(d_count, cstart.data(), sizeof(int32_t) * cstart.size(), cudaMemcpyHostToDevice);
    int32_t* d_cursor = dalloc<int32_t>((size_t)cells, own.v, e);
    if (e == cudaSuccess) e = cudaMemcpy(d_cursor, cstart.data(), sizeof(int32_t) * (size_t)cells, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (cells)", e);
        return NC_ERR_CUDA;
    }
    k_fill_cells<<<(n + 255) / 256, 256>>>(n, d_cell, d_cursor, d_members);
    k_knn<<<knn_blocks, 32 * kKnnWarps>>>(n, k, G.h, G.g, k0, k1, d_xyz, d_count, d_members, d_scratch, d_to, d_w,
                                          d_flags);
    uint32_t flags = 0;
    e = cudaMemcpy(&flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (search)", e);
        return NC_ERR_CUDA;
    }
    if (flags) {
        err = "device kNN build: candidate capacity exceeded";
        return NC_ERR_UNSUPPORTED;
    }
    // host description: positions, storage order, tables (no synapses yet)
    std::vector<float> xyz(3 * (size_t)n);
    e = cudaMemcpy(xyz.data(), d_xyz, sizeof(float) * xyz.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (positions)", e);
        return NC_ERR_CUDA;
    }
    NetHost& h = net->host;
    int rc = build_net(n, xyz.data(), 0, nullptr, nullptr, nullptr, nullptr, nullptr, p, h, err);
    if (rc != NC_OK) return rc;
    // h.nonneg_terms stays true: the weights written below are in [0, 1) and no synapse is
    // inhibitory, so no term of this network can be negative
    h.nonneg_terms = true;
    // in-degrees by target slot -> row starts
    int32_t* d_slot = dalloc<int32_t>((size_t)n, own.v, e);
    int32_t* d_deg = dalloc<int32_t>((size_t)n, own.v, e);
    if (e == cudaSuccess) e = cudaMemcpy(d_slot, h.slot_of.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_deg, 0, sizeof(int32_t) * (size_t)n);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (rows)", e);
        return NC_ERR_CUDA;
    }
    const unsigned eb = (unsigned)((edges + 255) / 256);
    k_indegree<<<eb, 256>>>(edges, d_to, d_slot, d_deg);
    std::vector<int32_t> deg((size_t)n);
    e = cudaMemcpy(deg.data(), d_deg, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (degrees)", e);
        return NC_ERR_CUDA;
    }
    h.in_ptr.assign((size_t)n + 1, 0);
    for (int32_t j = 0; j < n; ++j) h.in_ptr[(size_t)j + 1] = h.in_ptr[(size_t)j] + deg[(size_t)j];
    h.s = edges;
    h.n_input = edges;
    h.max_delay = 1;
    // device pools; the synapse streams are written below
    std::vector<const NetHost*> nets{&h};
    rc = net->eng.build(nets, 64, err, nullptr, true);
    if (rc != NC_OK) return rc;
    unsigned long long* d_cur = dalloc<unsigned long long>((size_t)n, own.v, e);
    unsigned long long* d_rows = dalloc<unsigned long long>((size_t)edges, own.v, e);
    int64_t* d_i2c = dalloc<int64_t>((size_t)edges, own.v, e);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_cur, h.in_ptr.data(), sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (scatter)", e);
        return e == cudaErrorMemoryAllocation ? NC_ERR_NOMEM : NC_ERR_CUDA;
    }
    k_scatter_rows<<<eb, 256>>>(edges, k, d_to, d_slot, d_cur, d_rows);
    k_fill_rows<<<std::max(1, sms * 8), 32 * kRowWarps>>>(net->eng.P, n, k, h.dt, d_xyz, d_to, d_w, d_slot, d_rows,
                                                          d_i2c, d_flags);
    e = cudaMemcpy(&flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = cuda_msg("device kNN build (rows)", e);
        return NC_ERR_CUDA;
    }
    if (flags & kFlagDelay) {
        err = "synapse delay exceeds 16383 steps";
        return NC_ERR_INVALID;
    }
    if (flags) {
        err = "device kNN build: row capacity exceeded";
        return NC_ERR_UNSUPPORTED;
    }
    // read-back tables stay on the device until a read-back asks for them
    net->dev_to = d_to;
    net->dev_i2c = d_i2c;
    own.v.erase(std::remove(own.v.begin(), own.v.end(), (void*)d_to), own.v.end());
    own.v.erase(std::remove(own.v.begin(), own.v.end(), (void*)d_i2c), own.v.end());
    net->knn_k = k;
    return NC_OK;
}

}  // namespace nc
