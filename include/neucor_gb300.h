/*
 * neucor_gb300.h — C ABI of the GB300 NeuroCorrelation simulation step.
 *
 * The reference exposes its simulator as the C++ class NeuCor (src/NeuCor.h:36-138)
 * with no C ABI.  Each entry point below replaces one member of that class (cited
 * beside it); include/neucor_gb300.hpp wraps them back into a class with the
 * reference's method names.
 *
 * Model.  A handle holds one network resident in GPU memory and advances it in
 * fixed steps of run_speed ms, every neuron updated every step — the reference's
 * NeuCor::run with runAll=true (src/NeuCor.cpp:583-617, 595-597).  Spike delays are
 * rounded to whole steps.  Within a step the reference's per-object rules are
 * applied in ascending neuron-id order (the stepped model; the parity tests compare
 * against a CPU restatement of it and against the reference's own code).
 *
 * Conventions.  Every function returns NC_OK (0) or a negative NC_ERR_* code; the
 * message of the calling thread's last error is nc_last_error().  No C++ exception
 * crosses this boundary.  Arrays are caller-owned host buffers unless stated.  Calls
 * on one handle must be serialised by the caller; distinct handles may be used from
 * distinct threads.  Every handle owns one CUDA stream.
 */
#ifndef NEUCOR_GB300_H
#define NEUCOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NC_OK 0
#define NC_ERR_INVALID (-1)     /* bad argument */
#define NC_ERR_CUDA (-2)        /* CUDA runtime error (message in nc_last_error) */
#define NC_ERR_NOMEM (-3)       /* device or host allocation failed */
#define NC_ERR_UNSUPPORTED (-4) /* reference operation outside the stepped GPU model */
#define NC_ERR_NODEVICE (-5)    /* no CUDA device */
#define NC_ERR_TIMEOUT (-6)     /* a bounded device-side wait gave up */
#define NC_ERR_BUDGET (-7)      /* request does not fit the memory budget */

typedef struct nc_net nc_net;

/* Synapse::inhibitory (src/NeuCor.h:290) selects the weight clamp of plasticity
 * (src/NeuCor.cpp:760-761).  setWeight sets it from the sign (src/NeuCor.cpp:576-579),
 * but the Synapse copy constructor (src/NeuCor.cpp:487-504) does not copy it, so a
 * synapse copied when its source's outSynapses vector grows (reserve(5),
 * src/NeuCor.cpp:374, then capacity doubling) carries an indeterminate flag.
 *   NC_INHIBITORY_COPY_LOSS  copied synapses are not inhibitory — what the reference
 *                            shows when the grown vector lands in fresh memory (default);
 *   NC_INHIBITORY_SIGN       inhibitory = weight < 0 for every synapse.
 * An explicit flag array given to nc_create overrides the rule. */
#define NC_INHIBITORY_COPY_LOSS 0
#define NC_INHIBITORY_SIGN 1

/* Simulation constants.  Field meanings follow NeuCor's public members
 * (src/NeuCor.h:68-73, defaults src/NeuCor.cpp:18-29). */
typedef struct {
    float run_speed;                /* NeuCor::runSpeed: ms per step; fixed for the handle's life */
    float learning_rate;            /* NeuCor::learningRate */
    float presynaptic_trace_decay;  /* copied into each Synapse at construction (src/NeuCor.cpp:464) */
    float postsynaptic_trace_decay; /* copied into each Neuron at construction (src/NeuCor.cpp:369) */
    float presynaptic_factor;       /* NeuCor::presynapticFactor */
    float postsynaptic_factor;      /* NeuCor::postsynapticFactor */
    int32_t background_firing;      /* 1: random background fires every step (src/NeuCor.cpp:604-607); 0: off */
    int32_t inhibitory_rule;        /* NC_INHIBITORY_* below */
    uint64_t seed;                  /* key of the counter-based draws (background, inputs) */
    int32_t storage_order;          /* NC_ORDER_*: how neurons are laid out in device memory */
    int32_t step_mode;              /* NC_STEP_*: which form of the step kernels runs */
} nc_params;

/* Device layout of neurons.  Results never depend on it (ids, the in-synapse fold
 * order and the same-step order rules all use the caller's ids).
 *   NC_ORDER_SPATIAL  Morton order of the positions (default): a neuron's targets sit
 *                     near it in memory, so the scattered accesses of a step share cache
 *                     lines;
 *   NC_ORDER_ID       the caller's id order. */
#define NC_ORDER_SPATIAL 0
#define NC_ORDER_ID 1

/* Form of the step kernels.  Results never depend on it.
 *   NC_STEP_DENSE  (default) two launches per step: a synapse pass that streams every
 *                  in-synapse row in order, making the launch decisions, the plasticity
 *                  and the arrival window there, and a neuron pass.  Its cost grows with
 *                  the synapse count: the faster form when a large share of neurons fires
 *                  every step.
 *   NC_STEP_EVENT  two launches per step; fired neurons are compacted into a list and
 *                  only their out-synapses and the arrived spikes are touched.  Its cost
 *                  grows with the synaptic events: the faster form for sparse activity.
 *   NC_STEP_AUTO   a single network (nc_create, nc_create_knn) holds the tables of both
 *                  forms and switches between them at run-call boundaries from the share
 *                  of neurons that fired in the last window of steps (see nc_run); the
 *                  switch keeps every bit of the state.  It costs the memory of both forms.
 * Networks batched into one engine (nc_batch_create) run in the first network's form
 * (dense or event). */
#define NC_STEP_DENSE 0
#define NC_STEP_EVENT 1
#define NC_STEP_AUTO 2

/* A group of input neurons driven by Poisson spike trains.  Members are the
 * neurons first .. first+count-1.  Correlated groups share one source whose every
 * event reaches each member jittered by a uniform +-jitter steps; independent
 * groups give each member its own train.  A member's spike is a forced fire
 * request (Neuron::scheduleFire, src/NeuCor.cpp:658-661, 682-686). */
typedef struct {
    int32_t first;
    int32_t count;
    float rate_hz;
    int32_t correlated;
    int32_t jitter;
} nc_group;

/* Counters of a handle since creation. */
typedef struct {
    int64_t steps;     /* steps simulated */
    int64_t fires;     /* neuron spikes */
    int64_t launched;  /* synaptic events: spikes accepted by a synapse (src/NeuCor.cpp:727-738) */
    int64_t dropped;   /* spikes a busy synapse refused (src/NeuCor.cpp:728) */
} nc_stats;

/* Render snapshot of one synapse: NeuCor::SynapseSnapshot (src/NeuCor.h:45-54,
 * src/NeuCor.cpp:115-134). */
typedef struct {
    int32_t from_id;
    int32_t to_id;
    float weight;
    float pre_potential;   /* Synapse::getPrePot, src/NeuCor.cpp:551-558 */
    float post_potential;  /* Synapse::getPostPot, src/NeuCor.cpp:560-567 */
    int32_t inhibitory;
} nc_synapse_snapshot;

/* One periodic input firer: NeuCor::InputSnapshot (src/NeuCor.h:56-62,
 * src/NeuCor.cpp:136-152). */
typedef struct {
    int32_t id;
    float x, y, z;       /* InputFirer::a */
    float radius;        /* InputFirer::radius */
    float frequency;     /* its entry of the rate array (0 past the array's end), Hz */
    int32_t enabled;     /* InputFirer::enabled: always 1 (the reference never clears it) */
} nc_input_snapshot;

/* ---------------------------------------------------------------- errors */
const char* nc_last_error(void);
const char* nc_version(void);
/* Number of usable CUDA devices (0 on a machine without a GPU). */
int nc_device_count(int* count);
/* Makes `device` the calling thread's current device; nc_create places a network on
 * the current device. */
int nc_set_device(int device);

/* ------------------------------------------------------------ lifecycle */
/* Defaults of NeuCor::NeuCor (src/NeuCor.cpp:18-29); background on, seed 0. */
int nc_default_params(nc_params* out);

/* Builds a network from explicit neurons and synapses on the current CUDA device.
 * Replaces NeuCor(0) + createNeuron(position) per neuron + createSynapse(to, from,
 * weight) per synapse, in the given order (src/NeuCor.cpp:17-42, 154-195).  A repeated
 * (from, to) pair keeps its first weight, as createSynapse does.  syn_length may be
 * NULL: lengths are then coord3::getDist of the endpoint positions (src/NeuCor.h:16-18,
 * src/NeuCor.cpp:477-479).  A spike takes length*2 ms (src/NeuCor.cpp:485,733), rounded
 * to whole steps, at least one.  syn_inhibitory may be NULL (flags then follow
 * params->inhibitory_rule). */
int nc_create(int32_t n_neurons, const float* xyz, int64_t n_synapses, const int32_t* syn_from,
              const int32_t* syn_to, const float* syn_weight, const float* syn_length,
              const uint8_t* syn_inhibitory, const nc_params* params, nc_net** out);
/* Frees the handle and its device memory (NeuCor::~NeuCor, src/NeuCor.cpp:44). */
int nc_destroy(nc_net* net);

/* Poisson input groups (replaces the role of NeuCor::setInputRateArray,
 * src/NeuCor.cpp:46-64, with the correlated trains of the benchmark workloads). */
int nc_set_input_groups(nc_net* net, int32_t n_groups, const nc_group* groups);
/* Periodic input firers (NeuCor::setInputRateArray, src/NeuCor.cpp:46-64, and
 * InputFirer, src/NeuCor.cpp:305-345).  Firers are appended or removed from the end to
 * match `count`; the i-th appended firer sits at xyz[3i..3i+2] with radius[i] (both
 * NULL: a random position from the C library's rand(), as the reference, and radius
 * 1).  rates_hz[i] is firer i's frequency (the reference re-reads its borrowed array
 * every run; here the rates are copied: change them with nc_set_input_rates).  Each
 * firer keeps the reference's schedule (lastFire + k*1000/f, float/double arithmetic):
 * step t evaluates it for the run call at currentTime T_t, the float sum of t
 * run_speeds, and a fire time inside (T_t, T_t + run_speed) fires every neuron closer
 * than the radius at step t+1 with Neuron::fire's semantics (no threshold or refractory
 * test); a firer set before the first step also meets the call at time 0, whose fires
 * land in step 1.  Changes take effect at the next step, as they do at the next run in
 * the reference.  Like the reference, with an exactly representable run_speed a period
 * of a whole number of steps never fires unless shifted with nc_add_input_offset. */
int nc_set_input_rate_array(nc_net* net, const float* rates_hz, uint32_t count, const float* xyz,
                            const float* radius);
/* New frequencies of the first `count` firers (the reference's borrowed rate array). */
int nc_set_input_rates(nc_net* net, int32_t count, const float* rates_hz);
/* NeuCor::addInputOffset (src/NeuCor.cpp:66-68): shifts firer `id`'s lastFire by t ms. */
int nc_add_input_offset(nc_net* net, int32_t id, float t_ms);
/* NeuCor::setDetectors (src/NeuCor.cpp:70-77): appends `count` voltage detectors at
 * xyz[3i..] with radius[i] (NULL: random positions from rand(), radius 1). */
int nc_set_detectors(nc_net* net, int32_t count, const float* xyz, const float* radius);
/* NeuCor::getDetectorVoltages / getDetectorVoltage (src/NeuCor.cpp:79-87, 359-366): the
 * mean potential of each detector's neurons (float sum in id order; NaN with no neuron
 * in range), as of the last completed step.  *count receives the detector count. */
int nc_get_detector_voltages(nc_net* net, float* out, int32_t capacity, int32_t* count);
int nc_get_detector_voltage(nc_net* net, int32_t id, float* out);
/* Runtime-settable rates (NeuCor::learningRate, presynapticFactor,
 * postsynapticFactor are read live by the reference, src/NeuCor.cpp:757-758). */
int nc_set_rates(nc_net* net, float learning_rate, float presynaptic_factor, float postsynaptic_factor);
/* Forced fire requests for the next step (Neuron::scheduleFire, src/NeuCor.cpp:658-661). */
int nc_schedule_fire(nc_net* net, int32_t count, const int32_t* neuron_ids);

/* ------------------------------------------------------------------ run */
/* Advances n_steps steps (NeuCor::run called n_steps times, src/NeuCor.cpp:583-617).
 * Asynchronous on the handle's stream; read-backs synchronise.  A network in
 * NC_STEP_AUTO runs in windows of NC_AUTO_WINDOW steps (a window may span several run
 * calls) and reads its fire count at the end of each (a synchronisation): it moves to
 * the event form when fewer than
 * NC_AUTO_TO_EVENT_PERMILLE per mille of its neurons fired per step in the window, and
 * back to the dense form above NC_AUTO_TO_DENSE_PERMILLE (the measured crossover of the
 * two forms on a 100k-neuron, 100-fan-out network lies between). */
#define NC_AUTO_WINDOW 256
#define NC_AUTO_TO_EVENT_PERMILLE 100
#define NC_AUTO_TO_DENSE_PERMILLE 160
int nc_run(nc_net* net, int32_t n_steps);
/* The form the network's next steps run in (NC_STEP_DENSE or NC_STEP_EVENT).  A network
 * created with NC_STEP_AUTO may be switched by the caller with nc_set_step_form (form
 * NC_STEP_DENSE or NC_STEP_EVENT pins it, NC_STEP_AUTO hands the choice back to nc_run);
 * other networks accept only their own form.  No counterpart in the reference. */
int nc_get_step_form(nc_net* net, int32_t* form);
int nc_set_step_form(nc_net* net, int32_t form);
/* Waits for the handle's queued work. */
int nc_sync(nc_net* net);
/* NeuCor::getTime (src/NeuCor.cpp:225): simulated ms, accumulated in float like the
 * reference. */
int nc_get_time(nc_net* net, float* ms);
int nc_get_step(nc_net* net, int64_t* step);
int nc_get_counts(nc_net* net, int32_t* n_neurons, int64_t* n_synapses);

/* Records the spike raster of the next max_steps steps into device memory
 * (replaces the renderer's per-frame scan of Neuron::lastFire,
 * src/NeuCor_Renderer.cpp:1841-1870).  max_steps = 0 stops recording. */
int nc_record_raster(nc_net* net, int32_t max_steps);
/* Copies the recorded raster: steps rows of ceil(N/8) bytes, bit j of row r set
 * when neuron j fired at the r-th recorded step.  *steps receives the row count. */
int nc_read_raster(nc_net* net, uint8_t* out, int64_t capacity_bytes, int32_t* steps);

/* ------------------------------------------------------------ read-back */
/* NeuCor::potAct (src/NeuCor.h:105): potential, activity interleaved, 2*N floats. */
int nc_read_potact(nc_net* net, float* out_2n);
int nc_read_potentials(nc_net* net, float* out_n);
/* NeuCor::positions (src/NeuCor.h:104), 3*N floats. */
int nc_read_positions(nc_net* net, float* out_3n);
/* Neuron::lastFire (src/NeuCor.h:226) in ms, NaN when the neuron never fired. */
int nc_read_last_fire(nc_net* net, float* out_n);
/* Synapse weights (Synapse::getWeight, src/NeuCor.cpp:572) in the order the
 * synapses were given to nc_create; NaN for ignored duplicates. */
int nc_read_weights(nc_net* net, float* out_s);
/* Delay of each synapse in steps, same order; -1 for ignored duplicates. */
int nc_read_delays(nc_net* net, int32_t* out_s);
/* Synapse::inhibitory of each synapse, same order: 0/1, 255 for ignored duplicates. */
int nc_read_inhibitory(nc_net* net, uint8_t* out_s);
/* NeuCor::getSynapseSnapshots (src/NeuCor.cpp:115-134), one entry per kept
 * synapse in source-then-creation order (the reference's outSynapses order). */
int nc_read_synapse_snapshots(nc_net* net, nc_synapse_snapshot* out, int64_t capacity, int64_t* count);
/* NeuCor::getInputSnapshots (src/NeuCor.cpp:136-152): one record per periodic input firer,
 * in firer order.  *count receives the number of firers; out may be NULL to query it. */
int nc_read_input_snapshots(nc_net* net, nc_input_snapshot* out, int32_t capacity, int32_t* count);
/* NeuCor::resetActivities (src/NeuCor.cpp:233-235). */
int nc_reset_activities(nc_net* net);
int nc_get_stats(nc_net* net, nc_stats* out);

/* Topology mutation after construction (NeuCor::deleteNeuron / deleteSynapse /
 * queFlip, src/NeuCor.cpp:230-232, 265-296) is outside the GPU model:
 * these return NC_ERR_UNSUPPORTED. */
int nc_delete_synapse(nc_net* net, int32_t from_id, int32_t to_id);
int nc_delete_neuron(nc_net* net, int32_t id);

/* ------------------------------------------------------ network builders */
/* Host-side construction helpers (no GPU needed).
 *
 * nc_build_knn: n neurons uniform in a cube of side (n/density)^(1/3), each
 * connected to its k nearest neighbours (ties by index), weights uniform [0,1),
 * all drawn from the counter-based generator keyed by seed.  Outputs: xyz (3n),
 * from/to/weight (n*k).  Lengths follow coord3::getDist (src/NeuCor.h:16-18). */
int nc_build_knn(int32_t n, int32_t k, float density, uint64_t seed, float* xyz, int32_t* syn_from,
                 int32_t* syn_to, float* syn_weight);
/* The network nc_build_knn describes, passed to nc_create — built on the GPU instead:
 * positions, the grid-hash neighbour search, weights and the in-synapse rows are
 * computed on the device (identical bits: same draws, same distances, same (distance,
 * id) order, same rows).  Dense form only (params->step_mode = NC_STEP_DENSE; an event-
 * form request, or one past the device builder's capacities — k > 512, more than 16,384
 * neighbour candidates or 2,048 in-synapses per neuron — is built on the host).
 * xyz_out (3n floats, may be NULL) receives the positions. */
int nc_create_knn(int32_t n, int32_t k, float density, uint64_t seed, const nc_params* params, float* xyz_out,
                  nc_net** out);
/* The reference constructor NeuCor(n) (src/NeuCor.cpp:17-42) in three calls that draw
 * from the C library's rand() in the reference's order, so after srand(s) they build
 * the network the reference builds after srand(s):
 *   nc_reference_positions: createNeuron with random positions in a sphere
 *     (src/NeuCor.cpp:154-170), 3*n floats (draws rand());
 *   nc_reference_connection_count: pairs closer than 1 unit (src/NeuCor.cpp:418-444),
 *     no draws;
 *   nc_reference_connections: those pairs in the reference's order with weights
 *     rand()*0.8+0.2, 20% negated (src/NeuCor.cpp:471-473) (draws rand()). */
int nc_reference_positions(int32_t n, float* xyz);
int nc_reference_connection_count(int32_t n, const float* xyz, int64_t* n_synapses);
int nc_reference_connections(int32_t n, const float* xyz, int32_t* syn_from, int32_t* syn_to, float* syn_weight,
                             int64_t capacity);

/* Philox4x32-10 (Salmon et al., SC'11), the counter-based generator behind every draw. */
int nc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ------------------------------------------------------ batched networks */
/* Many independent networks packed into one device engine and advanced together:
 * every launch pair steps every unfinished network once.  Each network keeps its own
 * constants, seed, inputs and horizon, and no state is shared, so a network computes
 * the same bits alone (nc_create) or packed.  There is no reference counterpart: the
 * reference simulates one NeuCor at a time (src/NeuCor.cpp:583-617). */
typedef struct nc_batch nc_batch;

typedef struct {
    int32_t n_neurons;
    const float* xyz;            /* 3*n; may be NULL if syn_length is given */
    int64_t n_synapses;
    const int32_t* syn_from;
    const int32_t* syn_to;
    const float* syn_weight;
    const float* syn_length;     /* may be NULL */
    const uint8_t* syn_inhibitory; /* may be NULL */
    nc_params params;
    int32_t n_groups;
    const nc_group* groups;
    int32_t horizon;             /* steps to simulate; the network idles afterwards */
} nc_net_spec;

/* Launch configuration of an engine (the autotuner's search space). */
typedef struct {
    int32_t neuron_block;        /* threads per block of the neuron update, or of the dense step
                                    (32..256, multiple of 32) */
    int32_t launch_blocks;       /* event form: blocks of the spike launch */
    int32_t launch_block;        /* event form: threads per block of the spike launch (32..256) */
    int32_t graph_steps;         /* steps per captured CUDA graph */
    int32_t dense_blocks;        /* dense form: blocks of the synapse pass (a grid-stride loop over
                                    256-synapse spans); 0 = one wave of resident blocks */
    int32_t steps_per_launch;    /* dense form: 0 = each step is two launches (replayed through CUDA
                                    graphs of graph_steps steps); k > 0 = k whole steps per
                                    persistent cooperative launch (grid barriers between the
                                    passes; networks with periodic input firers use graphs) */
} nc_launch_config;

int nc_batch_create(int32_t n_nets, const nc_net_spec* specs, nc_batch** out);
int nc_batch_destroy(nc_batch* batch);
/* Advances every unfinished network by up to `steps` steps. */
int nc_batch_run(nc_batch* batch, int32_t steps);
/* Same, timed with CUDA events on the engine's stream (ms of device time). */
int nc_batch_time(nc_batch* batch, int32_t steps, float* ms);
/* Runs until every network reached its horizon. */
int nc_batch_run_to_end(nc_batch* batch);
int nc_batch_get_launch(nc_batch* batch, nc_launch_config* out);
int nc_batch_set_launch(nc_batch* batch, const nc_launch_config* cfg);
/* Times `steps_per_trial` steps under each candidate configuration, three times each
 * after a warm-up trial, and keeps the one with the lowest median; *best receives it.
 * The candidates cover block sizes, the synapse pass's grid, graph length and (dense
 * form) steps per persistent launch.  The simulation advances during the trials; the
 * results do not depend on the configuration. */
int nc_batch_autotune(nc_batch* batch, int32_t steps_per_trial, nc_launch_config* best);
int nc_batch_get_stats(nc_batch* batch, int32_t net, nc_stats* out);
int nc_batch_get_step(nc_batch* batch, int32_t net, int64_t* step);
int nc_batch_read_potentials(nc_batch* batch, int32_t net, float* out_n);
int nc_batch_read_weights(nc_batch* batch, int32_t net, float* out_s);
int nc_batch_read_last_fire(nc_batch* batch, int32_t net, float* out_n);

/* ---------------------------------------------------------- served form */
/* A request server: simulation jobs (networks with their own size, inputs and
 * horizon) are submitted while others run; each is admitted when its device
 * footprint fits the memory budget and a slot is free, stays resident on the device
 * while it runs, and leaves when it reaches its horizon.  Networks admitted at
 * different times advance together in the same launches (continuous batching); each
 * computes the same bits it would alone.  No reference counterpart: the reference
 * simulates one NeuCor at a time. */
typedef struct nc_server nc_server;

typedef struct {
    int64_t memory_budget_bytes; /* device memory for resident networks */
    int32_t max_networks;        /* networks resident at once */
    int32_t steps_per_batch;     /* steps between admission / completion decisions */
    int32_t build_threads;       /* host threads preparing submitted networks; they pause while the
                                    prepared, not yet admitted requests hold more than 8 GiB of
                                    host tables */
    int32_t keep_results;        /* 1: keep finished networks' weights and potentials for nc_server_fetch */
    int32_t step_mode;           /* NC_STEP_*: form of the step kernels for every request */
} nc_server_config;

typedef struct {
    int64_t request_id;
    int32_t status;    /* NC_OK, or why the request was refused (NC_ERR_BUDGET, NC_ERR_INVALID) */
    int32_t n_neurons;
    int32_t horizon;
    int32_t reserved;
    int64_t n_synapses;
    double submit_s;   /* seconds since the server started */
    double admit_s;
    double done_s;
    nc_stats stats;
} nc_request_done;

typedef struct {
    int64_t submitted, admitted, finished, rejected;
    int64_t resident_bytes;      /* footprint of the networks resident now */
    int64_t peak_resident_bytes;
    int64_t peak_resident_networks;
    int64_t steps_run;           /* launch pairs issued */
    double device_busy_s;        /* device time of the step batches */
} nc_server_stats;

int nc_server_create(const nc_server_config* config, nc_server** out);
/* Copies the spec's arrays; returns at once.  NC_ERR_BUDGET if the network could never
 * fit the budget. */
int nc_server_submit(nc_server* server, const nc_net_spec* spec, int64_t* request_id);
/* A request for the kNN network nc_build_knn(n, k, density, knn_seed) describes (the
 * workloads' networks), built by one of the server's builder threads: the caller sends
 * parameters only, and the network's arrays exist only while that thread prepares it.
 * No counterpart in the reference. */
int nc_server_submit_knn(nc_server* server, int32_t n, int32_t k, float density, uint64_t knn_seed,
                         const nc_params* params, int32_t n_groups, const nc_group* groups, int32_t horizon,
                         int64_t* request_id);
/* Finished requests since the last poll (at most `capacity`). */
int nc_server_poll(nc_server* server, nc_request_done* out, int32_t capacity, int32_t* count);
/* Blocks until every submitted request has finished. */
int nc_server_drain(nc_server* server);
/* Final weights (creation order, as nc_read_weights) and potentials of a finished
 * request, when the server keeps results; either pointer may be NULL.  Releases them. */
int nc_server_fetch(nc_server* server, int64_t request_id, float* weights, float* potentials);
int nc_server_get_stats(nc_server* server, nc_server_stats* out);
int nc_server_destroy(nc_server* server);

/* Advances the network like nc_run, for callers that cannot let the library allocate
 * device memory once the network exists: a simulation service that reserves a fixed
 * device-memory budget up front and admits work against it, or a host program (a
 * renderer, a game or robotics engine embedding the simulator) whose own allocator owns
 * the GPU's memory.  For them a cudaMalloc made behind their back can fail when the
 * memory is spoken for, or break their accounting.  nc_run instantiates CUDA graphs on
 * first use and, in the event form (NC_STEP_EVENT), keeps its per-step scratch (the
 * list of neurons that fired, passed from the neuron update to the spike launch) in
 * memory the handle allocated.  This call launches the same kernels directly on
 * `stream` (NULL = the handle's own stream) and calls no cudaMalloc, cudaFree or
 * allocating library routine.  The dense form needs no scratch; the event form uses a
 * fixed scratch array compiled into the library.  That array (4 MiB) is held by every
 * GPU that loads the library until the process exits, and it limits event-form calls
 * to networks of at most NC_NOALLOC_MAX_NEURONS neurons; larger ones are refused with
 * NC_ERR_INVALID.  The first event-form call on a device looks the array's device
 * address up (cudaGetSymbolAddress) and keeps it; make that first call before any
 * stream capture.  Every call clears the array's counters before its kernels run; the
 * array otherwise keeps the last call's contents, and all event-form calls share it,
 * so calls whose kernels overlap on the GPU (other handles, other streams) race: order
 * them.  Order the call after the handle's earlier work, and synchronise `stream`
 * before any other call on the handle when it is not the handle's stream.  After this
 * call the handle reads its step counter and simulated time back from the device
 * (nc_get_step, nc_get_time and the read-backs wait for the handle's stream to do so).
 * The reference has no counterpart: its simulator runs on the CPU and allocates
 * nothing on a GPU. */
#define NC_NOALLOC_MAX_NEURONS 262144
int nc_run_noalloc(nc_net* net, int32_t n_steps, void* stream);

/* Times n_steps of the handle's step kernels with CUDA events on its stream;
 * *ms receives the elapsed device time, *kernel_ms (may be NULL) two entries:
 * the mean time of one neuron-update and one spike-launch launch over a separate
 * instrumented pass of min(n_steps, 200) steps (dense form: the synapse pass and the
 * neuron pass). */
int nc_time_steps(nc_net* net, int32_t n_steps, float* ms, float* kernel_ms);

#ifdef __cplusplus
}
#endif
#endif
