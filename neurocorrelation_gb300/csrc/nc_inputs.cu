// nc_inputs.cu — periodic input firers and voltage detectors on the device.
//
// InputFirer (src/NeuCor.cpp:305-345): at every NeuCor::run the firer schedules the fire
// times lastFire + k*1000/frequency that fall in (currentT, currentT + runSpeed), and
// when one comes up it calls Neuron::fire() on every neuron closer than its radius — a
// fire with no threshold and no refractory test.  In the stepped model step t is the
// run call that starts at currentTime T_t (the float sum of t runSpeeds, as the
// reference keeps it): k_input_firers runs that call's schedule before the step's
// kernels — after any change the caller made before it, as in the reference — and a
// fire inside (T_t, T_t + runSpeed) fires the near neurons at step t+1.  Before the
// first step it also runs the call at time 0, whose fires land in step 1.  The
// schedule's float/double arithmetic is the reference's, so its behaviour carries over,
// including that with an exactly representable step a period of a whole number of steps
// never fires (its `currentT < fireTime` test excludes the boundary).
//
// VoltageDetector::getVoltage (src/NeuCor.cpp:359-366): the mean potential of the
// neurons closer than the detector's radius, summed in id order in float.
#include "nc_engine.cuh"

#include <cuda_runtime.h>

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int32_t kFirerLoopCap = 1 << 20;  // schedule passes per firer and step

// InputFirer::schedule(deltaT, frequency) at currentT; returns whether a fire time fell
// in (currentT, currentT + deltaT).  *capped: the pass cap was reached (the reference
// would loop without end when the period does not advance fireTime).
__device__ bool firer_schedule(float* last, float dt, float frequency, float currentT, bool* capped)
{
    bool fired = false;
    *capped = false;
    if (frequency == 0.0f) return false;
    if (*last != *last) *last = 0.0f;  // lastFire = 0 when NaN
    const double period = __ddiv_rn(1000.0, (double)frequency);
    const float end = __fadd_rn(currentT, dt);
    int32_t pass = 0;
    for (float fireTime = __double2float_rn(__dadd_rn((double)*last, period)); fireTime < end;
         fireTime = __double2float_rn(__dadd_rn((double)fireTime, period))) {
        if (pass++ >= kFirerLoopCap) {
            *capped = true;
            break;
        }
        if (currentT < fireTime) {
            fired = true;
            *last = fireTime;
        }
    }
    return fired;
}

__device__ void mark_near(const NcPools& P, const NcFirer& F, uint32_t* uf, int lane)
{
    for (int32_t k = F.near_begin + lane; k < F.near_end; k += 32) {
        const int32_t slot = P.firer_near[k];
        atomicOr(uf + (slot >> 5), 1u << (slot & 31));
    }
}

// Warp per firer, before the kernels of its net's step t = D.t: lane 0 runs the
// schedule, the warp marks the near neurons.
__global__ void k_input_firers(NcPools P)
{
    const int lane = threadIdx.x & 31;
    const int f = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (f >= P.n_firers) return;
    NcFirer& F = P.firers[f];
    const NcNetDesc& D = P.nets[F.net];
    if (!D.active || D.t > D.t_end) return;
    int fired0 = 0, fired = 0;
    if (lane == 0) {
        float last = F.last;
        bool capped = false, capped0 = false;
        // the run call at time 0 (D.tsum = 0 before the first step): fires at step 1
        if (F.first && D.t == 1) fired0 = firer_schedule(&last, D.dt, F.rate, D.tsum, &capped0) ? 1 : 0;
        // the call starting at T_t = T_{t-1} + runSpeed (currentTime = targetTime)
        fired = firer_schedule(&last, D.dt, F.rate, __fadd_rn(D.tsum, D.dt), &capped) ? 1 : 0;
        F.last = last;
        F.first = 0;
        if (capped || capped0) atomicOr(P.dev_err, NC_DEV_ERR_FIRER_LOOP);
    }
    fired0 = __shfl_sync(kFull, fired0, 0);
    fired = __shfl_sync(kFull, fired, 0);
    uint32_t* uf = P.ufire + D.word_base;
    if (fired0) mark_near(P, F, uf + (int64_t)(D.t & 1) * P.total_words, lane);
    if (fired) mark_near(P, F, uf + (int64_t)((D.t + 1) & 1) * P.total_words, lane);
}

// Thread per detector: mean potential of its near neurons (caller ids, ascending).
__global__ void k_detector_voltages(const float* pot, const int32_t* slot_of, int32_t neuron_base, const int32_t* near,
                                    const int32_t* near_ptr, int32_t count, float* out)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= count) return;
    float avg = 0.0f;
    const int32_t b = near_ptr[d], e = near_ptr[d + 1];
    for (int32_t k = b; k < e; ++k) avg = __fadd_rn(avg, pot[neuron_base + slot_of[neuron_base + near[k]]]);
    out[d] = __fdiv_rn(avg, (float)(uint32_t)(e - b));  // avgV / near.size()
}

}  // namespace

namespace nc {

int launch_input_firers(const NcPools& P, void* stream)
{
    if (P.n_firers <= 0) return 0;
    const int threads = 256;
    const int blocks = (int)(((int64_t)P.n_firers * 32 + threads - 1) / threads);
    k_input_firers<<<blocks, threads, 0, (cudaStream_t)stream>>>(P);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_detector_voltages(const NcPools& P, int32_t neuron_base, const int32_t* near, const int32_t* near_ptr,
                             int32_t count, float* out, void* stream)
{
    if (count <= 0) return 0;
    k_detector_voltages<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(P.pot, P.slot_of, neuron_base, near,
                                                                             near_ptr, count, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace nc
