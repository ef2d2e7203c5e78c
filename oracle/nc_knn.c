/* nc_knn.c — the workloads' k-nearest-neighbour networks, restated on the CPU.
 *
 * TEST INFRASTRUCTURE (part of the oracle, with nc_oracle.c): builds the same network as the
 * library's nc_build_knn / nc_create_knn from the definition alone, so that fixtures,
 * the CPU baseline and the reference arm of the benchmark can make the workloads'
 * networks without loading the library under test.
 *
 * The network (not the reference's own sphere construction, src/NeuCor.cpp:17-42,
 * 154-170: the workloads ask for cubes with k nearest targets, made through the
 * reference's createNeuron/createSynapse, src/NeuCor.cpp:154-195):
 *   side      = (float)cbrt((double)n / (double)density)
 *   xyz[i][a] = unit24(o[a]) * side, o = Philox4x32-10(i, 0, 10, 0; seed)
 *   targets   = the k points j != i with the smallest (getDist(i, j), j), ascending;
 *               getDist is coord3::getDist (src/NeuCor.h:16-18): sqrtf of the float
 *               sum dx*dx + dy*dy + dz*dz
 *   weight[m] = unit24(o[m & 3]), o = Philox4x32-10(i, m >> 2, 11, 0; seed)
 *   unit24(r) = (r >> 8) * 2^-24
 * Synapses are listed by source, then by rank m.
 *
 * The search is exact: a uniform grid of cells of side h, visited in shells of growing
 * Chebyshev radius r around the point's cell.  A point outside shells 0..r lies more
 * than r*h away along some axis, so the search stops once the k-th best distance is
 * below (r - 1/1024) * h (the margin covers the float rounding of cell indices).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "nc_oracle.h"

static float unit24(uint32_t r) { return (float)(r >> 8) * 0x1p-24f; }

static float dist3(const float* a, const float* b)
{
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

typedef struct {
    int32_t n, k, g;
    float h;
    const float* xyz;
    const int32_t* cstart;   /* g^3 + 1 */
    const int32_t* members;
    int32_t* to;
    int32_t next;            /* next point to take (under mu) */
    pthread_mutex_t mu;
} knn_job;

static int32_t cell1(float v, float h, int32_t g)
{
    int32_t c = (int32_t)(v / h);
    return c < 0 ? 0 : (c >= g ? g - 1 : c);
}

/* keeps best[0..cnt) sorted by (d, j); inserts (d, j) if it belongs to the k best */
static void offer(float* bd, int32_t* bj, int32_t* cnt, int32_t k, float d, int32_t j)
{
    int32_t c = *cnt;
    if (c == k) {
        if (d > bd[k - 1] || (d == bd[k - 1] && j > bj[k - 1])) return;
        c = k - 1;
    }
    int32_t p = c;
    while (p > 0 && (bd[p - 1] > d || (bd[p - 1] == d && bj[p - 1] > j))) {
        bd[p] = bd[p - 1];
        bj[p] = bj[p - 1];
        --p;
    }
    bd[p] = d;
    bj[p] = j;
    if (*cnt < k) *cnt += 1;
}

static void* knn_worker(void* arg)
{
    knn_job* J = (knn_job*)arg;
    const int32_t k = J->k, g = J->g;
    float* bd = (float*)malloc(sizeof(float) * (size_t)k);
    int32_t* bj = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int32_t lo = J->next;
        J->next += 256;
        pthread_mutex_unlock(&J->mu);
        if (lo >= J->n) break;
        const int32_t hi = lo + 256 < J->n ? lo + 256 : J->n;
        for (int32_t i = lo; i < hi; ++i) {
            const float* pi = J->xyz + 3 * (size_t)i;
            const int32_t cx = cell1(pi[0], J->h, g), cy = cell1(pi[1], J->h, g), cz = cell1(pi[2], J->h, g);
            int32_t cnt = 0;
            for (int32_t r = 0; r <= g; ++r) {
                for (int32_t x = cx - r; x <= cx + r; ++x) {
                    if (x < 0 || x >= g) continue;
                    for (int32_t y = cy - r; y <= cy + r; ++y) {
                        if (y < 0 || y >= g) continue;
                        const int edge_xy = (x == cx - r || x == cx + r || y == cy - r || y == cy + r);
                        for (int32_t z = cz - r; z <= cz + r; z += (edge_xy || r == 0) ? 1 : 2 * r) {
                            if (z < 0 || z >= g) continue;
                            const int32_t c = (x * g + y) * g + z;
                            for (int32_t q = J->cstart[c]; q < J->cstart[c + 1]; ++q) {
                                const int32_t j = J->members[q];
                                if (j != i) offer(bd, bj, &cnt, k, dist3(pi, J->xyz + 3 * (size_t)j), j);
                            }
                        }
                    }
                }
                if (cnt == k && bd[k - 1] < ((float)r - 1.0f / 1024.0f) * J->h) break;
            }
            memcpy(J->to + (size_t)i * k, bj, sizeof(int32_t) * (size_t)k);
        }
    }
    free(bd);
    free(bj);
    return NULL;
}

int ncs_build_knn(int32_t n, int32_t k, float density, uint64_t seed, int32_t threads, float* xyz,
                  int32_t* syn_from, int32_t* syn_to, float* syn_weight)
{
    if (n < 0 || k < 0 || !(density > 0.0f) || !xyz) return -1;
    if (n > 0 && k >= n) return -1;
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const float side = (float)cbrt((double)n / (double)density);
    for (int32_t i = 0; i < n; ++i) {
        const uint32_t ctr[4] = {(uint32_t)i, 0u, 10u, 0u};
        uint32_t o[4];
        ncs_philox4x32_10(ctr, key, o);
        for (int a = 0; a < 3; ++a) xyz[3 * (size_t)i + a] = unit24(o[a]) * side;
    }
    if (n == 0 || k == 0) return 0;
    /* cells holding about four points each */
    int32_t g = (int32_t)floor((double)side / cbrt(4.0 / (double)density));
    if (g < 1) g = 1;
    if (g > 512) g = 512;
    const float h = side / (float)g;
    const size_t ncell = (size_t)g * g * g;
    int32_t* cstart = (int32_t*)calloc(ncell + 1, sizeof(int32_t));
    int32_t* cell = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* members = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!cstart || !cell || !members) { free(cstart); free(cell); free(members); return -2; }
    for (int32_t i = 0; i < n; ++i) {
        const float* p = xyz + 3 * (size_t)i;
        cell[i] = (cell1(p[0], h, g) * g + cell1(p[1], h, g)) * g + cell1(p[2], h, g);
        cstart[cell[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; ++c) cstart[c + 1] += cstart[c];
    {
        int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * ncell);
        memcpy(fill, cstart, sizeof(int32_t) * ncell);
        for (int32_t i = 0; i < n; ++i) members[fill[cell[i]]++] = i;  /* ascending id within a cell */
        free(fill);
    }
    knn_job J = {n, k, g, h, xyz, cstart, members, syn_to, 0, PTHREAD_MUTEX_INITIALIZER};
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    int started = 0;
    for (int32_t t = 1; t < threads; ++t)
        if (pthread_create(&th[started], NULL, knn_worker, &J) == 0) started++;
    knn_worker(&J);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(cstart);
    free(cell);
    free(members);
    for (int32_t i = 0; i < n; ++i) {
        for (int32_t m = 0; m < k; ++m) {
            const size_t q = (size_t)i * k + m;
            syn_from[q] = i;
            const uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(m >> 2), 11u, 0u};
            uint32_t o[4];
            ncs_philox4x32_10(ctr, key, o);
            syn_weight[q] = unit24(o[m & 3]);
        }
    }
    return 0;
}
