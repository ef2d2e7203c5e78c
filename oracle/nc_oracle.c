/*
 * Oracle-S — CPU restatement of the NeuCor simulation step (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm load this file's library.  It is the oracle, never the product.
 *
 * Every function below names the reference lines it restates.  Arithmetic is
 * kept in the reference's own types: float state, double where the reference
 * mixes in double literals or exp(), libm powf/exp called at the same points.
 * Compile with -ffp-contract=off so no multiply-add is fused (the reference's
 * x86-64 build has no FMA either).
 *
 * Time: step t is time T = t*dt.  The reference keeps float times; for the
 * step sizes used here (dyadic dt, e.g. 1 ms) every time and time difference is
 * exact, and a difference of k steps is the float k*dt.
 *
 * Same-step ordering.  Within one time T the reference runs its events in heap
 * order, which leaves two outcomes open:
 *   (i)  a synapse whose spike arrived at T-KC*dt is freed by its target's
 *        update at T (NeuCor.cpp:697) -- a launch at T by its source
 *        (NeuCor.cpp:728) succeeds only if that update ran first;
 *   (ii) when source and target both fire at T, the target's post-spike
 *        plasticity (NeuCor.cpp:651-653) may or may not precede the weight
 *        capture of the source's launch (NeuCor.cpp:729-731).
 * The oracle fixes both by running neuron updates in ascending id order, each
 * update doing its whole fire() at once, then the arrivals of time T.  Both
 * coincidences are counted (ncs_stats.order_conflicts) so comparisons against
 * the heap-ordered reference know how far they may expect bit equality.
 */
#include "nc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NEVER INT32_MIN
#define FREE_SLOT INT32_MIN

/* ---------------------------------------------------------------- Philox */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
 * as 1, 2, 3" (SC'11).  Multipliers and Weyl key increments from that paper. */
void ncs_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0;
        c1 = (uint32_t)p1;
        c2 = n2;
        c3 = (uint32_t)p0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static uint32_t draw(const uint32_t key[2], uint32_t a, uint32_t b, uint32_t stream, uint32_t c, int lane)
{
    uint32_t ctr[4] = {a, b, stream, c}, out[4];
    ncs_philox4x32_10(ctr, key, out);
    return out[lane];
}

/* Draw streams (third counter word). */
enum { STREAM_BACKGROUND = 1, STREAM_SOURCE = 2, STREAM_JITTER = 3, STREAM_INDEPENDENT = 4 };

/* ----------------------------------------------------------------- state */
struct ncs_net {
    int32_t n;
    int64_t s;            /* synapses kept (duplicates dropped) */
    int64_t n_input;      /* synapses given */
    ncs_params p;
    float dt;
    int32_t kc;           /* smallest k with AP_cutoff(2.0f) < k*dt */
    int32_t bg_period;    /* max(1, int(600/dt)), NeuCor.cpp:605 */

    /* CSC: in-synapses of each target, ascending source id (std::map order, NeuCor.h:212) */
    int64_t* post_ptr;
    int32_t* pre;
    int32_t* post;
    int32_t* delay;
    int64_t* out_ptr;     /* per source: its synapses' CSC indices */
    int64_t* out_syn;
    int64_t* input_to_csc;/* input synapse k -> CSC index or -1 (duplicate) */

    /* Synapse state (NeuCor.h:282-293) */
    float* w;
    uint8_t* inh;
    float* depol;         /* AP_depolFac captured at launch */
    int32_t* arr;         /* AP_fireTime as a step; FREE_SLOT when 0 in the reference */
    int32_t* t_arr;       /* lastSpikeArrival as a step; NEVER = -INFINITY */
    int32_t* launch_step; /* diagnostics for order conflicts */
    int32_t* stdp_step;

    /* Neuron state (NeuCor.h:226-241) */
    float* pot;
    float* activity;
    int32_t* lf;          /* lastFire as a step; NEVER = NaN */
    uint32_t* firings;
    int32_t* act_start;   /* activityStartTime as a step */
    int32_t* busy;        /* in-synapses not FREE, to skip idle neurons */
    uint8_t* forced;      /* requests for step cur+1 (scheduledFireTime == T) */
    uint8_t* ufire;       /* InputFirer fires for step cur+1 (Neuron::fire, no threshold) */
    uint8_t* ufire_next;  /* ... for step cur+2 */
    float* xyz;           /* neuron positions (NeuCor::positions) */
    float tsum;           /* NeuCor::currentTime at the start of step cur's run call: the
                             float sum of cur runSpeeds (NeuCor.cpp:616) */

    /* periodic input firers (InputFirer, NeuCor.cpp:305-345) */
    int32_t n_firers;
    float* f_last;        /* InputFirer::lastFire, ms */
    float* f_rate;        /* the firer's entry of the rate array, Hz */
    int64_t* f_ptr;       /* near lists: f_ids[f_ptr[i] .. f_ptr[i+1]) */
    uint8_t* f_first;     /* set before the first step: the run call at time 0 evaluates it too */
    int32_t* f_ids;

    /* arrivals bucketed by step modulo ring */
    int32_t ring;
    int64_t** bucket;
    int64_t* bucket_len;
    int64_t* bucket_cap;

    int32_t n_groups;
    ncs_group* groups;
    uint32_t* group_thresh;

    int32_t cur;
    ncs_stats st;
};

void ncs_default_params(ncs_params* p)
{
    /* NeuCor::NeuCor, NeuCor.cpp:18-29 */
    memset(p, 0, sizeof(*p));
    p->run_speed = 1.0f;
    p->learning_rate = 1.0f;
    p->presynaptic_trace_decay = 0.75f;
    p->postsynaptic_trace_decay = 0.65f;
    p->presynaptic_factor = 0.13f;
    p->postsynaptic_factor = 0.30f;
    p->background_firing = 1;
    p->inhibitory_rule = NCS_INHIBITORY_COPY_LOSS;
    p->seed = 0;
}

/* Whether the m-th synapse (0-based) appended to an outSynapses vector of final size
 * `size` was copied by a reallocation: the vector is reserved to 5 (NeuCor.cpp:374)
 * and libstdc++ doubles its capacity when full. */
static int grown_copy(int64_t m, int64_t size)
{
    int64_t cap = 5;
    while (cap <= m) cap *= 2;
    return size > cap;
}

static float kdt(const ncs_net* h, int32_t k) { return (float)k * h->dt; }
static int32_t background_period(float dt);
static void draw_background(ncs_net* h, int32_t counter);

/* coord3::getDist, NeuCor.h:16-18 (GCC folds powf(x,2) to x*x). */
static float get_dist(const float* a, const float* b)
{
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

/* Delay in steps of a spike travelling length*AP_speed ms (NeuCor.cpp:485,733),
 * rounded to the nearest step, at least one step. */
static int32_t delay_steps(float length, float dt)
{
    float ms = length * 2.0f;
    float q = floorf(ms / dt + 0.5f);
    if (!(q >= 1.0f)) return 1;
    if (q > 32767.0f) return -1;
    return (int32_t)q;
}

static uint32_t rate_threshold(float rate_hz, float dt)
{
    double prob = (double)rate_hz * (double)dt / 1000.0;
    if (!(prob > 0.0)) return 0;
    double v = prob * 4294967296.0;
    if (v >= 4294967295.0) return 4294967295u;
    return (uint32_t)v;
}

static void* xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz ? sz : 1); }

typedef struct { int32_t post, pre; int64_t idx; } key3;

static int cmp_key3(const void* a, const void* b)
{
    const key3* x = (const key3*)a;
    const key3* y = (const key3*)b;
    if (x->post != y->post) return x->post < y->post ? -1 : 1;
    if (x->pre != y->pre) return x->pre < y->pre ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

ncs_net* ncs_create(int32_t n, const float* xyz, int64_t n_syn, const int32_t* syn_pre,
                    const int32_t* syn_post, const float* syn_weight, const float* syn_length,
                    const uint8_t* syn_inhibitory, const ncs_params* params)
{
    if (n < 0 || n_syn < 0 || !params) return NULL;
    if (!(params->run_speed > 0.0f)) return NULL;
    if (n_syn > 0 && (!syn_pre || !syn_post || !syn_weight)) return NULL;
    if (n_syn > 0 && !syn_length && !xyz) return NULL;
    for (int64_t k = 0; k < n_syn; ++k)
        if (syn_pre[k] < 0 || syn_pre[k] >= n || syn_post[k] < 0 || syn_post[k] >= n) return NULL;

    ncs_net* h = (ncs_net*)xcalloc(1, sizeof(ncs_net));
    h->n = n;
    h->n_input = n_syn;
    h->p = *params;
    h->xyz = (float*)xcalloc((size_t)n * 3, sizeof(float));  /* positions, for the firers' near lists */
    if (xyz) memcpy(h->xyz, xyz, sizeof(float) * 3 * (size_t)n);
    h->dt = params->run_speed;
    h->kc = 1;
    while (!(2.0f < kdt(h, h->kc))) h->kc++;
    h->bg_period = background_period(h->dt);

    /* Sort by (target, source); createSynapse keeps the first of duplicates
     * (NeuCor.cpp:189-191). */
    key3* keys = (key3*)xcalloc((size_t)n_syn, sizeof(key3));
    for (int64_t k = 0; k < n_syn; ++k) {
        keys[k].post = syn_post[k];
        keys[k].pre = syn_pre[k];
        keys[k].idx = k;
    }
    qsort(keys, (size_t)n_syn, sizeof(key3), cmp_key3);
    h->input_to_csc = (int64_t*)xcalloc((size_t)n_syn, sizeof(int64_t));
    for (int64_t k = 0; k < n_syn; ++k) h->input_to_csc[k] = -1;
    int64_t s = 0;
    for (int64_t k = 0; k < n_syn; ++k) {
        if (k > 0 && keys[k].post == keys[k - 1].post && keys[k].pre == keys[k - 1].pre) continue;
        keys[s++] = keys[k];
    }
    h->s = s;
    h->post_ptr = (int64_t*)xcalloc((size_t)n + 1, sizeof(int64_t));
    h->pre = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->post = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->delay = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->w = (float*)xcalloc((size_t)s, sizeof(float));
    h->inh = (uint8_t*)xcalloc((size_t)s, 1);
    h->depol = (float*)xcalloc((size_t)s, sizeof(float));
    h->arr = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->t_arr = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->launch_step = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    h->stdp_step = (int32_t*)xcalloc((size_t)s, sizeof(int32_t));
    int32_t max_delay = 1;
    for (int64_t c = 0; c < s; ++c) {
        int64_t k = keys[c].idx;
        h->input_to_csc[k] = c;
        h->pre[c] = keys[c].pre;
        h->post[c] = keys[c].post;
        h->post_ptr[keys[c].post + 1]++;
        /* Synapse ctor + setWeight: weight, inhibitory = weight < 0 (NeuCor.cpp:475,576-579) */
        h->w[c] = syn_weight[k];
        h->inh[c] = syn_weight[k] < 0.0f;  /* replaced below for copied synapses */
        float len = syn_length ? syn_length[k]
                               : get_dist(&xyz[3 * (int64_t)keys[c].pre], &xyz[3 * (int64_t)keys[c].post]);
        int32_t d = delay_steps(len, h->dt);
        if (d < 0) { free(keys); ncs_destroy(h); return NULL; }
        h->delay[c] = d;
        if (d > max_delay) max_delay = d;
        h->arr[c] = FREE_SLOT;          /* AP_fireTime = 0 (NeuCor.cpp:484) */
        h->t_arr[c] = NEVER;            /* lastSpikeArrival = -INFINITY (NeuCor.cpp:469) */
        h->launch_step[c] = NEVER;
        h->stdp_step[c] = NEVER;
    }
    for (int32_t j = 0; j < n; ++j) h->post_ptr[j + 1] += h->post_ptr[j];
    free(keys);

    /* out-synapses of each source in creation order (Neuron::outSynapses) */
    h->out_ptr = (int64_t*)xcalloc((size_t)n + 1, sizeof(int64_t));
    h->out_syn = (int64_t*)xcalloc((size_t)s, sizeof(int64_t));
    for (int64_t c = 0; c < s; ++c) h->out_ptr[h->pre[c] + 1]++;
    for (int32_t j = 0; j < n; ++j) h->out_ptr[j + 1] += h->out_ptr[j];
    {
        int64_t* fill = (int64_t*)xcalloc((size_t)n + 1, sizeof(int64_t));
        for (int64_t k = 0; k < n_syn; ++k) {
            int64_t c = h->input_to_csc[k];
            if (c < 0) continue;
            int32_t i = h->pre[c];
            h->out_syn[h->out_ptr[i] + fill[i]++] = c;
        }
        free(fill);
    }
    if (params->inhibitory_rule == NCS_INHIBITORY_COPY_LOSS) {
        for (int32_t i = 0; i < n; ++i) {
            int64_t size = h->out_ptr[i + 1] - h->out_ptr[i];
            for (int64_t m = 0; m < size; ++m)
                if (grown_copy(m, size)) h->inh[h->out_syn[h->out_ptr[i] + m]] = 0;
        }
    }
    if (syn_inhibitory) {
        for (int64_t k = 0; k < n_syn; ++k)
            if (h->input_to_csc[k] >= 0) h->inh[h->input_to_csc[k]] = syn_inhibitory[k] ? 1 : 0;
    }

    /* Neuron ctor, NeuCor.cpp:368-395 */
    h->pot = (float*)xcalloc((size_t)n, sizeof(float));
    h->activity = (float*)xcalloc((size_t)n, sizeof(float));
    h->lf = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
    h->firings = (uint32_t*)xcalloc((size_t)n, sizeof(uint32_t));
    h->act_start = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
    h->busy = (int32_t*)xcalloc((size_t)n, sizeof(int32_t));
    h->forced = (uint8_t*)xcalloc((size_t)n, 1);
    h->ufire = (uint8_t*)xcalloc((size_t)n, 1);
    h->ufire_next = (uint8_t*)xcalloc((size_t)n, 1);
    for (int32_t j = 0; j < n; ++j) {
        h->pot[j] = -70.0f;   /* setPotential(baselevel) */
        h->activity[j] = 0.0f;
        h->lf[j] = NEVER;     /* lastFire = NAN */
    }

    h->ring = 1;
    while (h->ring < max_delay + 2) h->ring <<= 1;
    h->bucket = (int64_t**)xcalloc((size_t)h->ring, sizeof(int64_t*));
    h->bucket_len = (int64_t*)xcalloc((size_t)h->ring, sizeof(int64_t));
    h->bucket_cap = (int64_t*)xcalloc((size_t)h->ring, sizeof(int64_t));

    h->cur = 0;
    h->st.first_conflict_step = -1;
    h->st.step = 0;

    /* Step 0: every neuron's run at T=0 returns at once (deltaT == 0,
     * NeuCor.cpp:626); only the background draws for step 1 are made. */
    if (h->p.background_firing && n > 0) draw_background(h, 0);
    return h;
}

void ncs_destroy(ncs_net* h)
{
    if (!h) return;
    free(h->post_ptr); free(h->pre); free(h->post); free(h->delay); free(h->out_ptr);
    free(h->out_syn); free(h->input_to_csc); free(h->w); free(h->inh); free(h->depol);
    free(h->arr); free(h->t_arr); free(h->launch_step); free(h->stdp_step);
    free(h->pot); free(h->activity); free(h->lf); free(h->firings); free(h->act_start);
    free(h->busy); free(h->forced); free(h->ufire); free(h->ufire_next);
    free(h->f_last); free(h->f_rate); free(h->f_ptr); free(h->f_ids); free(h->f_first); free(h->xyz);
    if (h->bucket)
        for (int32_t r = 0; r < h->ring; ++r) free(h->bucket[r]);
    free(h->bucket); free(h->bucket_len); free(h->bucket_cap);
    free(h->groups); free(h->group_thresh);
    free(h);
}

int ncs_set_groups(ncs_net* h, int32_t n_groups, const ncs_group* groups)
{
    if (!h || n_groups < 0 || (n_groups > 0 && !groups)) return -1;
    for (int32_t g = 0; g < n_groups; ++g) {
        if (groups[g].first < 0 || groups[g].count < 0 || groups[g].jitter < 0 ||
            (int64_t)groups[g].first + groups[g].count > h->n)
            return -1;
    }
    free(h->groups);
    free(h->group_thresh);
    h->groups = (ncs_group*)xcalloc((size_t)n_groups, sizeof(ncs_group));
    h->group_thresh = (uint32_t*)xcalloc((size_t)n_groups, sizeof(uint32_t));
    memcpy(h->groups, groups, sizeof(ncs_group) * (size_t)n_groups);
    for (int32_t g = 0; g < n_groups; ++g) h->group_thresh[g] = rate_threshold(groups[g].rate_hz, h->dt);
    h->n_groups = n_groups;
    return 0;
}

int ncs_set_rates(ncs_net* h, float lr, float pre_factor, float post_factor)
{
    if (!h) return -1;
    h->p.learning_rate = lr;
    h->p.presynaptic_factor = pre_factor;
    h->p.postsynaptic_factor = post_factor;
    return 0;
}

int ncs_schedule_fire(ncs_net* h, int32_t count, const int32_t* ids)
{
    if (!h || count < 0) return -1;
    for (int32_t k = 0; k < count; ++k) {
        if (ids[k] < 0 || ids[k] >= h->n) return -1;
    }
    for (int32_t k = 0; k < count; ++k) h->forced[ids[k]] = 1;
    return 0;
}

/* Whether member m of group g requests a fire at step t.  Correlated groups
 * share one Poisson source; each source event at step s reaches member m at
 * s + jitter(s, m), jitter uniform in [-J, J].  Independent groups draw one
 * Bernoulli per member and step. */
static int group_member_fires(const ncs_group* gr, uint32_t g, uint32_t th, const uint32_t key[2],
                              uint32_t m, int32_t t)
{
    if (!gr->correlated) return draw(key, g, (uint32_t)t, STREAM_INDEPENDENT, m, 0) < th;
    int32_t jit = gr->jitter;
    for (int32_t src = t - jit; src <= t + jit; ++src) {
        if (src < 0) continue;
        if (!(draw(key, g, (uint32_t)src, STREAM_SOURCE, 0u, 0) < th)) continue;
        int32_t off = (int32_t)(draw(key, g, (uint32_t)src, STREAM_JITTER, m, 0) % (uint32_t)(2 * jit + 1)) - jit;
        if (src + off == t) return 1;
    }
    return 0;
}

static int input_request(const ncs_net* h, int32_t j, int32_t t)
{
    uint32_t key[2] = {(uint32_t)h->p.seed, (uint32_t)(h->p.seed >> 32)};
    for (int32_t g = 0; g < h->n_groups; ++g) {
        const ncs_group* gr = &h->groups[g];
        if (j < gr->first || j >= gr->first + gr->count) continue;
        if (group_member_fires(gr, (uint32_t)g, h->group_thresh[g], key, (uint32_t)(j - gr->first), t)) return 1;
    }
    return 0;
}

int32_t ncs_input_fires(const ncs_group* groups, int32_t n_groups, uint64_t seed, float dt, int32_t t,
                        int32_t* ids, int32_t cap)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    int32_t count = 0;
    for (int32_t g = 0; g < n_groups; ++g) {
        uint32_t th = rate_threshold(groups[g].rate_hz, dt);
        for (int32_t m = 0; m < groups[g].count; ++m) {
            if (!group_member_fires(&groups[g], (uint32_t)g, th, key, (uint32_t)m, t)) continue;
            if (count < cap) ids[count] = groups[g].first + m;
            count++;
        }
    }
    return count;
}

static int32_t background_period(float dt)
{
    int period = (int)(600.0f / dt);  /* std::max(1, static_cast<int>(600.0f / runSpeed)) */
    return period < 1 ? 1 : period;
}

void ncs_background_draws(uint64_t seed, int32_t n, float dt, int32_t counter, uint8_t* hit, int32_t* target)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t period = (uint32_t)background_period(dt);
    for (int32_t i = 0; i < n; ++i) {
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)counter, STREAM_BACKGROUND, 0u}, o[4];
        ncs_philox4x32_10(ctr, key, o);
        hit[i] = (o[0] % period) == 0;
        target[i] = (int32_t)(o[1] % (uint32_t)n);
    }
}

int32_t ncs_delay_steps(float length, float dt) { return delay_steps(length, dt); }

static void draw_background(ncs_net* h, int32_t counter)
{
    uint32_t key[2] = {(uint32_t)h->p.seed, (uint32_t)(h->p.seed >> 32)};
    uint32_t period = (uint32_t)h->bg_period;
    for (int32_t i = 0; i < h->n; ++i) {
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)counter, STREAM_BACKGROUND, 0u}, o[4];
        ncs_philox4x32_10(ctr, key, o);
        if (o[0] % period == 0) h->forced[o[1] % (uint32_t)h->n] = 1;
    }
}

/* Synapse::synapticPlasticity, NeuCor.cpp:740-761, with Neuron::getTrace
 * (NeuCor.cpp:671-675).  fmin/fmax keep C99's generic semantics. */
static void plasticity(ncs_net* h, int64_t c, int32_t t)
{
    int32_t target = h->post[c];
    float traceS = h->t_arr[c] == NEVER ? 0.0f
                                        : powf(h->p.presynaptic_trace_decay, kdt(h, t - h->t_arr[c]));
    float traceT = h->lf[target] == NEVER ? 0.0f
                                          : powf(h->p.postsynaptic_trace_decay, kdt(h, t - h->lf[target]));
    if (traceT == 1) traceT = 0;
    if (traceS == 1) traceS = 0;
    float weightChange = h->p.presynaptic_factor * traceS - h->p.postsynaptic_factor * traceT;
    float w = h->w[c];
    w += weightChange * h->p.learning_rate;
    if (!h->inh[c]) {
        float m = (w <= 1.0f) ? w : 1.0f;   /* fmin(weight, 1.0) */
        w = (m >= 0.0f) ? m : 0.0f;         /* fmax(.., 0.0) */
    } else {
        float m = (w <= 0.0f) ? w : 0.0f;
        w = (m >= -1.0f) ? m : -1.0f;
    }
    if (w != h->w[c]) h->stdp_step[c] = t;
    h->w[c] = w;
}

static void note_conflict(ncs_net* h, int32_t t)
{
    h->st.order_conflicts++;
    if (h->st.first_conflict_step < 0) h->st.first_conflict_step = t;
}

static void push_arrival(ncs_net* h, int32_t a, int64_t c)
{
    int32_t r = a & (h->ring - 1);
    if (h->bucket_len[r] == h->bucket_cap[r]) {
        int64_t cap = h->bucket_cap[r] ? 2 * h->bucket_cap[r] : 64;
        h->bucket[r] = (int64_t*)realloc(h->bucket[r], (size_t)cap * sizeof(int64_t));
        h->bucket_cap[r] = cap;
    }
    h->bucket[r][h->bucket_len[r]++] = c;
}

/* Neuron::fire, NeuCor.cpp:643-656, with Synapse::fire, NeuCor.cpp:727-738. */
static void fire(ncs_net* h, int32_t j, int32_t t)
{
    h->lf[j] = t;
    h->firings[j]++;
    h->st.fires++;
    const float c52 = (float)((double)0.2f * 52.0);  /* AP_depolFac = 0.2f; *= 52.0 */
    for (int64_t k = h->out_ptr[j]; k < h->out_ptr[j + 1]; ++k) {
        int64_t c = h->out_syn[k];
        int32_t target = h->post[c];
        if (h->launch_step[c] != NEVER && t - (h->launch_step[c] + h->delay[c]) == h->kc &&
            target != j)
            note_conflict(h, t);
        if (h->arr[c] != FREE_SLOT) {  /* if (AP_fireTime != 0) return; */
            h->st.dropped++;
            continue;
        }
        if (target < j && h->lf[target] == t && h->stdp_step[c] == t) note_conflict(h, t);
        h->depol[c] = c52 * h->w[c];   /* AP_depolFac *= weight */
        h->arr[c] = t + h->delay[c];   /* AP_fireTime = length*AP_speed + now */
        h->launch_step[c] = t;
        h->busy[target]++;
        push_arrival(h, h->arr[c], c);
        h->st.launched++;
    }
    for (int64_t c = h->post_ptr[j]; c < h->post_ptr[j + 1]; ++c) {
        plasticity(h, c, t);
        /* a source that already launched on this synapse this step captured
         * the weight before this change */
        if (h->pre[c] != j && h->launch_step[c] == t && h->stdp_step[c] == t) note_conflict(h, t);
    }
}

/* Neuron::AP, NeuCor.cpp:706-714; x = (float)currentT - lastFire. */
static float ap_value(float x)
{
    const float AP_h = 100.0f, AP_depolW = 0.3f, AP_polW = 0.6f, AP_deltaPol = 1.16f;
    const float AP_depolFac = 0.2f, AP_deltaStart = 1.0f, baselevel = -70.0f, threshold = -55.0f;
    float a = x - AP_deltaStart;
    float b = x - AP_deltaStart - AP_deltaPol;
    double v = AP_h * (exp(-(a * a) / (2.0 * AP_depolW * AP_depolW)) -
                       exp(-(b * b) / (2.0 * AP_polW * AP_polW)) * AP_depolFac) +
               baselevel + (threshold - baselevel) * fmax(1.0 - (double)x, 0.0);
    return (float)v;
}

/* Neuron::run at step t >= 1, NeuCor.cpp:619-641.  `input`: an InputFirer fired the
 * neuron in the interval before t (InputFirer::run -> Neuron::fire, NeuCor.cpp:
 * 326-331), which the stepped model places at t: no threshold or refractory test. */
static void neuron_run(ncs_net* h, int32_t j, int32_t t, int forced, int input)
{
    const float deltaT = h->dt;
    const float currentT = kdt(h, t);
    /* charge_insynapses, NeuCor.cpp:688-700 */
    float newPot = h->pot[j];
    if (h->busy[j]) {
        for (int64_t c = h->post_ptr[j]; c < h->post_ptr[j + 1]; ++c) {
            if (h->arr[c] == FREE_SLOT) continue;               /* AP_fireTime == 0 */
            float timeOffset = kdt(h, t - h->arr[c]);
            if (timeOffset <= 0.0f) continue;
            newPot += deltaT * h->depol[c] * 0.9943 * exp(0.3702 * deltaT);
            if (2.0f < timeOffset) {                            /* AP_cutoff < timeOffset */
                h->arr[c] = FREE_SLOT;
                h->busy[j]--;
            }
        }
    }
    h->pot[j] = newPot;
    /* charge_passive, NeuCor.cpp:677-680 */
    h->pot[j] = ((float)h->pot[j] - -70.0f) * powf(0.5f, deltaT) + -70.0f;
    /* charge_thresholdCheck, NeuCor.cpp:682-686 (vesicles never drop below 0) */
    if (input || ((-55.0f < h->pot[j] || forced) &&
                  (h->lf[j] == NEVER || 2.0f < kdt(h, t - h->lf[j]))))
        fire(h, j, t);
    /* AP, NeuCor.cpp:706-714 */
    if (!(h->lf[j] == NEVER || 2.0f < kdt(h, t - h->lf[j]))) h->pot[j] = ap_value(kdt(h, t - h->lf[j]));
    /* setActivity, NeuCor.cpp:640 */
    h->activity[j] = (float)(h->firings[j] / (((float)currentT - kdt(h, h->act_start[j])) / 10.0));
}

/* InputFirer::schedule(deltaT, frequency), NeuCor.cpp:333-345, at currentT = t*dt:
 * the fire times lastFire + k*1000/frequency that fall in (currentT, currentT+deltaT),
 * in the reference's float/double arithmetic.  Returns 1 if any falls there.  The loop
 * is capped (NCS_FIRER_LOOP_CAP passes); the reference loops without end when the
 * period does not advance fireTime. */
#define NCS_FIRER_LOOP_CAP (1 << 20)
static int firer_schedule(float* last, float dt, float frequency, float currentT)
{
    int fired = 0;
    if (frequency == 0.0f) return 0;
    if (*last != *last) *last = 0.0f;
    int32_t pass = 0;
    for (float fireTime = (float)((double)*last + 1000.0 / frequency);
         fireTime < currentT + dt && pass < NCS_FIRER_LOOP_CAP;
         fireTime = (float)((double)fireTime + 1000.0 / frequency), ++pass) {
        if (currentT < fireTime) {
            fired = 1;
            *last = fireTime;
        }
    }
    return fired;
}

/* The firers' schedule for the run call starting at currentT (NeuCor::run, NeuCor.cpp:
 * 599-602); fires go to `mark` (the step after that call's neuron updates). */
static void firers_schedule(ncs_net* h, float currentT, int first_only, uint8_t* mark)
{
    for (int32_t i = 0; i < h->n_firers; ++i) {
        if (first_only && !h->f_first[i]) continue;
        if (firer_schedule(&h->f_last[i], h->dt, h->f_rate[i], currentT))
            for (int64_t k = h->f_ptr[i]; k < h->f_ptr[i + 1]; ++k) mark[h->f_ids[k]] = 1;
    }
}

int ncs_set_firers(ncs_net* h, int32_t count, const float* rates, const float* xyz, const float* radius)
{
    if (!h || count < 0 || (count > 0 && (!xyz || !radius))) return -1;
    /* the first min(old, count) firers keep their state: setInputRateArray appends or
       pops at the end (NeuCor.cpp:46-64) */
    const int32_t keep = h->n_firers < count ? h->n_firers : count;
    uint8_t* first = (uint8_t*)xcalloc((size_t)count, 1);
    float* last = (float*)xcalloc((size_t)count, sizeof(float));  /* lastFire(0.0), NeuCor.cpp:311 */
    for (int32_t i = 0; i < count; ++i) {
        first[i] = i < keep ? h->f_first[i] : (uint8_t)(h->cur == 0);
        last[i] = i < keep ? h->f_last[i] : 0.0f;
    }
    free(h->f_last); free(h->f_rate); free(h->f_ptr); free(h->f_ids); free(h->f_first);
    h->n_firers = count;
    h->f_first = first;
    h->f_last = last;
    h->f_rate = (float*)xcalloc((size_t)count, sizeof(float));
    h->f_ptr = (int64_t*)xcalloc((size_t)count + 1, sizeof(int64_t));
    int64_t total = 0;
    for (int32_t i = 0; i < count; ++i)
        for (int32_t j = 0; j < h->n; ++j)
            if (get_dist(&h->xyz[3 * (int64_t)j], &xyz[3 * (int64_t)i]) < radius[i]) ++total;
    h->f_ids = (int32_t*)xcalloc((size_t)total, sizeof(int32_t));
    total = 0;
    /* near: every neuron closer than radius, in id order (NeuCor.cpp:323-327) */
    for (int32_t i = 0; i < count; ++i) {
        h->f_rate[i] = rates ? rates[i] : 0.0f;
        for (int32_t j = 0; j < h->n; ++j)
            if (get_dist(&h->xyz[3 * (int64_t)j], &xyz[3 * (int64_t)i]) < radius[i]) h->f_ids[total++] = j;
        h->f_ptr[i + 1] = total;
    }
    return 0;
}

int ncs_set_firer_rates(ncs_net* h, int32_t count, const float* rates)
{
    if (!h || count < 0 || count > h->n_firers) return -1;
    for (int32_t i = 0; i < count; ++i) h->f_rate[i] = rates[i];
    return 0;
}

/* NeuCor::addInputOffset, NeuCor.cpp:66-68 */
int ncs_add_firer_offset(ncs_net* h, int32_t id, float t)
{
    if (!h || id < 0 || id >= h->n_firers) return -1;
    h->f_last[id] += t;
    return 0;
}

int32_t ncs_n_firers(const ncs_net* h) { return h ? h->n_firers : 0; }
void ncs_read_firer_last(const ncs_net* h, float* out)
{
    memcpy(out, h->f_last, sizeof(float) * (size_t)h->n_firers);
}

int ncs_run(ncs_net* h, int32_t n_steps, uint8_t* raster, float* pot_trace)
{
    if (!h || n_steps < 0) return -1;
    const int64_t row = ((int64_t)h->n + 7) / 8;
    for (int32_t r = 0; r < n_steps; ++r) {
        int32_t t = h->cur + 1;
        /* the input firers' run calls: the one at time 0 before the first step (its fires
         * land at step 1), then the one starting at T_t (fires at step t+1), each at the
         * reference's accumulated currentTime (NeuCor.cpp:599-602, 616) */
        if (h->n_firers > 0) {
            if (t == 1) firers_schedule(h, h->tsum, 1, h->ufire);
            for (int32_t i = 0; i < h->n_firers; ++i) h->f_first[i] = 0;
            firers_schedule(h, h->tsum + h->dt, 0, h->ufire_next);
        }
        for (int32_t j = 0; j < h->n; ++j) {
            int forced = h->forced[j] || input_request(h, j, t);
            neuron_run(h, j, t, forced, h->ufire[j]);
        }
        { uint8_t* u = h->ufire; h->ufire = h->ufire_next; h->ufire_next = u; }
        memset(h->ufire_next, 0, (size_t)h->n);
        /* spikes arriving at T: Synapse::run, NeuCor.cpp:718-726 */
        int32_t slot = t & (h->ring - 1);
        for (int64_t q = 0; q < h->bucket_len[slot]; ++q) {
            int64_t c = h->bucket[slot][q];
            h->t_arr[c] = t;               /* lastSpikeArrival = now */
            plasticity(h, c, t);
            h->st.arrivals++;
        }
        h->bucket_len[slot] = 0;
        /* background fires for step t+1, NeuCor.cpp:604-607 */
        memset(h->forced, 0, (size_t)h->n);
        if (h->p.background_firing && h->n > 0) draw_background(h, t);
        h->tsum = h->tsum + h->dt;  /* currentTime = targetTime (NeuCor.cpp:616) */
        if (raster) {
            uint8_t* rr = raster + (int64_t)r * row;
            memset(rr, 0, (size_t)row);
            for (int32_t j = 0; j < h->n; ++j)
                if (h->lf[j] == t) rr[j >> 3] |= (uint8_t)(1u << (j & 7));
        }
        if (pot_trace) memcpy(pot_trace + (int64_t)r * h->n, h->pot, sizeof(float) * (size_t)h->n);
        h->cur = t;
        h->st.step = t;
    }
    return 0;
}

int32_t ncs_step(const ncs_net* h) { return h ? h->cur : -1; }
int64_t ncs_n_synapses(const ncs_net* h) { return h ? h->s : -1; }

void ncs_read_potentials(const ncs_net* h, float* out) { memcpy(out, h->pot, sizeof(float) * (size_t)h->n); }
void ncs_read_activity(const ncs_net* h, float* out) { memcpy(out, h->activity, sizeof(float) * (size_t)h->n); }
void ncs_read_last_fire_step(const ncs_net* h, int32_t* out) { memcpy(out, h->lf, sizeof(int32_t) * (size_t)h->n); }

void ncs_read_weights(const ncs_net* h, float* out)
{
    for (int64_t k = 0; k < h->n_input; ++k) out[k] = h->input_to_csc[k] < 0 ? NAN : h->w[h->input_to_csc[k]];
}

void ncs_read_inhibitory(const ncs_net* h, uint8_t* out)
{
    for (int64_t k = 0; k < h->n_input; ++k) out[k] = h->input_to_csc[k] < 0 ? 255 : h->inh[h->input_to_csc[k]];
}

void ncs_read_delays(const ncs_net* h, int32_t* out)
{
    for (int64_t k = 0; k < h->n_input; ++k) out[k] = h->input_to_csc[k] < 0 ? -1 : h->delay[h->input_to_csc[k]];
}

/* NeuCor::resetActivities -> Neuron::resetActivity, NeuCor.cpp:233-235,460 */
void ncs_reset_activities(ncs_net* h)
{
    for (int32_t j = 0; j < h->n; ++j) {
        h->firings[j] = 0;
        h->act_start[j] = h->cur;
        h->activity[j] = 0.0f;
    }
}

void ncs_get_stats(const ncs_net* h, ncs_stats* out) { *out = h->st; }
