/*
 * Oracle-S: the CPU restatement of NeuroCorrelation's simulation step, used as
 * TEST INFRASTRUCTURE ONLY (the parity oracle for the CUDA path and the timed
 * CPU port in bench.py).  Nothing in the shipped library links or calls it.
 *
 * It follows the reference's per-object code in src/NeuCor.cpp expression by
 * expression (file:line citations in nc_oracle.c), driven by a fixed-dt stepped
 * scheduler instead of the reference's event heap:
 *
 *   every step t >= 1 (time T = t*dt), neurons in ascending id:
 *     Neuron::run  (NeuCor.cpp:619-641)  charge_insynapses -> charge_passive ->
 *                  charge_thresholdCheck -> (fire: Synapse::fire on out-synapses,
 *                  synapticPlasticity on in-synapses) -> AP
 *   then every spike arriving at T:  Synapse::run (NeuCor.cpp:718-726)
 *   then the background draws that schedule fires for step t+1 (NeuCor.cpp:604-607).
 *
 * With runAll=true, runSpeed=dt and synapse delays on the step grid this is what
 * the reference itself computes; the canonical ascending-id order resolves the
 * two same-step orderings the reference leaves to its heap (see nc_oracle.c).
 * The oracle is pinned against the reference's own code compiled from its
 * sources (oracle/_ref, built by oracle/Makefile) in tests/test_oracle_pin.py.
 */
#ifndef NC_ORACLE_H
#define NC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ncs_net ncs_net;

typedef struct {
    float run_speed;                /* NeuCor::runSpeed, ms per step (NeuCor.h:68) */
    float learning_rate;            /* NeuCor::learningRate (NeuCor.h:71) */
    float presynaptic_trace_decay;  /* copied into every Synapse at construction (NeuCor.cpp:464) */
    float postsynaptic_trace_decay; /* copied into every Neuron at construction (NeuCor.cpp:369) */
    float presynaptic_factor;       /* NeuCor.h:73 */
    float postsynaptic_factor;
    int32_t background_firing;      /* 1: NeuCor.cpp:604-607 background fires; 0: off */
    int32_t inhibitory_rule;        /* NCS_INHIBITORY_* (see below) */
    uint64_t seed;                  /* Philox key for background and input draws */
} ncs_params;

/* Synapse::inhibitory (NeuCor.h:290) is set from the weight's sign by setWeight
 * (NeuCor.cpp:576-579), but the Synapse copy constructor (NeuCor.cpp:487-504) does not
 * copy it: a synapse copied when its source's outSynapses vector grows (reserve(5),
 * NeuCor.cpp:374, then capacity doubling) reads an indeterminate flag.
 *   NCS_INHIBITORY_COPY_LOSS: copied synapses are not inhibitory (the value the
 *     reference shows when the grown vector lands in fresh memory);
 *   NCS_INHIBITORY_SIGN: inhibitory = weight < 0 for every synapse.
 * Explicit per-synapse flags passed to ncs_create override the rule. */
#define NCS_INHIBITORY_COPY_LOSS 0
#define NCS_INHIBITORY_SIGN 1

typedef struct {
    int32_t first;        /* first neuron id of the group */
    int32_t count;        /* members are neurons first .. first+count-1 */
    float rate_hz;        /* Poisson rate of the source (correlated) or of each member */
    int32_t correlated;   /* 1: members share one source, each spike jittered; 0: independent */
    int32_t jitter;       /* +-jitter steps around each shared source event */
} ncs_group;

typedef struct {
    int64_t fires;          /* neurons that fired */
    int64_t launched;       /* accepted synaptic launches (= deliveries) */
    int64_t dropped;        /* launches dropped because the synapse was busy (NeuCor.cpp:728) */
    int64_t arrivals;       /* spikes delivered */
    int64_t order_conflicts;     /* same-step coincidences whose outcome depends on event order */
    int32_t first_conflict_step; /* -1 if none */
    int32_t step;                /* last processed step */
} ncs_stats;

void ncs_default_params(ncs_params* p);

/* Builds a network from explicit neurons and synapses (NeuCor::createNeuron /
 * createSynapse, NeuCor.cpp:154-195).  syn_length may be NULL: lengths are then
 * coord3::getDist of the endpoints (NeuCor.h:16-18, NeuCor.cpp:477-479).
 * syn_inhibitory may be NULL: flags then follow params->inhibitory_rule.
 * Returns NULL on bad input. */
ncs_net* ncs_create(int32_t n_neurons, const float* xyz, int64_t n_syn,
                    const int32_t* syn_pre, const int32_t* syn_post,
                    const float* syn_weight, const float* syn_length,
                    const uint8_t* syn_inhibitory, const ncs_params* params);
/* Effective inhibitory flag of every input synapse (0/1; 255 for duplicates). */
void ncs_read_inhibitory(const ncs_net* h, uint8_t* out);
void ncs_destroy(ncs_net* h);

int ncs_set_groups(ncs_net* h, int32_t n_groups, const ncs_group* groups);
int ncs_set_rates(ncs_net* h, float learning_rate, float pre_factor, float post_factor);
/* Requests a forced fire (Neuron::scheduleFire, NeuCor.cpp:658-661) for the next step. */
int ncs_schedule_fire(ncs_net* h, int32_t n, const int32_t* ids);
/* Periodic input firers (NeuCor::setInputRateArray, InputFirer, NeuCor.cpp:46-64,
 * 305-345): firer i at xyz[3i..] fires every neuron closer than radius[i] at the
 * reference's schedule for rates[i] Hz.  At its start step t evaluates the run call at
 * the reference's currentTime T_t (the float sum of t runSpeeds): a fire time inside
 * (T_t, T_t + runSpeed) fires those neurons at step t+1, without threshold or
 * refractory test (Neuron::fire).  Step 1 also evaluates the call at time 0 for the
 * firers set before it, whose fires land in step 1.  Changes are seen by the next step.
 * xyz and radius give all `count` firers; the first min(previous, count) keep their
 * state (setInputRateArray appends and pops at the end). */
int ncs_set_firers(ncs_net* h, int32_t count, const float* rates, const float* xyz, const float* radius);
int ncs_set_firer_rates(ncs_net* h, int32_t count, const float* rates);
int ncs_add_firer_offset(ncs_net* h, int32_t id, float t);
int32_t ncs_n_firers(const ncs_net* h);
void ncs_read_firer_last(const ncs_net* h, float* out);  /* InputFirer::lastFire, ms */

/* Runs n steps.  raster (may be NULL): n * ceil(N/8) bytes, bit j of row r set
 * when neuron j fired at step cur+1+r.  pot_trace (may be NULL): n * N floats. */
int ncs_run(ncs_net* h, int32_t n_steps, uint8_t* raster, float* pot_trace);

int32_t ncs_step(const ncs_net* h);
int64_t ncs_n_synapses(const ncs_net* h);
void ncs_read_potentials(const ncs_net* h, float* out);
void ncs_read_activity(const ncs_net* h, float* out);
void ncs_read_last_fire_step(const ncs_net* h, int32_t* out); /* INT32_MIN = never */
void ncs_read_weights(const ncs_net* h, float* out);          /* input order; NaN for duplicates */
void ncs_read_delays(const ncs_net* h, int32_t* out);         /* input order */
void ncs_reset_activities(ncs_net* h);
void ncs_get_stats(const ncs_net* h, ncs_stats* out);

/* Philox4x32-10 (Salmon et al., SC'11), exported for known-answer tests. */
void ncs_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Input generation shared by the oracle and the reference harness, so both
 * see the same input spikes.  ncs_input_fires lists the group members that
 * request a fire at step t (returns the count, at most cap written). */
int32_t ncs_input_fires(const ncs_group* groups, int32_t n_groups, uint64_t seed, float dt,
                        int32_t t, int32_t* ids, int32_t cap);
/* Background draws made at step `counter` for step counter+1: hit[i] and
 * target[i] for every source i (NeuCor.cpp:604-607 with a counter-based RNG). */
void ncs_background_draws(uint64_t seed, int32_t n, float dt, int32_t counter, uint8_t* hit,
                          int32_t* target);
/* Delay in steps for a synapse of the given length (see nc_oracle.c). */
int32_t ncs_delay_steps(float length, float dt);

/* The workloads' kNN network (nc_knn.c): positions (3n floats) and n*k synapses by
 * source then rank; the same network as the library's nc_build_knn.  0 on success. */
int ncs_build_knn(int32_t n, int32_t k, float density, uint64_t seed, int32_t threads, float* xyz,
                  int32_t* syn_from, int32_t* syn_to, float* syn_weight);

#ifdef __cplusplus
}
#endif
#endif
