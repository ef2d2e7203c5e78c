// neucor_gb300.hpp — header-only C++ class with the reference's NeuCor interface
// (src/NeuCor.h:36-138) over the C ABI of neucor_gb300.h.
//
// A program written against the reference's class keeps its calls:
//
//     neucor_gb300::NeuCor brain(0);
//     brain.runAll = true; brain.runSpeed = 1.0f;
//     brain.createNeuron({0, 0, 0}); ...; brain.createSynapse(1, 0, 0.5f);
//     while (...) { brain.run(); auto snaps = brain.getNeuronSnapshots(); }
//
// The network is built on the GPU at the first run() (or read-back); after that the
// topology is fixed.  Public members are pushed to the device before every run(), as
// the reference reads them live.  Errors from the C ABI are thrown as
// neucor_gb300::Error (this header is C++ and may throw; the C ABI never does).
#ifndef NEUCOR_GB300_HPP
#define NEUCOR_GB300_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "neucor_gb300.h"

namespace neucor_gb300 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc)
{
    if (rc != NC_OK) throw Error(rc, nc_last_error());
}

// coord3 (src/NeuCor.h:13-24)
struct coord3 {
    float x, y, z;
    float getDist(coord3 c) const { return std::sqrt((x - c.x) * (x - c.x) + (y - c.y) * (y - c.y) + (z - c.z) * (z - c.z)); }
};

class NeuCor {
public:
    struct NeuronSnapshot {       // src/NeuCor.h:38-43
        std::size_t id;
        coord3 position;
        float potential;
        float activity;
    };
    struct SynapseSnapshot {      // src/NeuCor.h:45-54
        std::size_t fromID;
        std::size_t toID;
        coord3 from;
        coord3 to;
        float weight;
        float prePotential;
        float postPotential;
        bool inhibitory;
    };

    // NeuCor(int n_neurons) (src/NeuCor.cpp:17-42): n > 0 builds the reference's random
    // sphere network, drawing from the C library's rand() in the reference's order (seed
    // it with srand() first, as with the reference).
    explicit NeuCor(int n_neurons)
    {
        nc_params p;
        check(nc_default_params(&p));
        runSpeed = p.run_speed;
        runAll = false;
        learningRate = p.learning_rate;
        presynapticTraceDecay = p.presynaptic_trace_decay;
        postsynapticTraceDecay = p.postsynaptic_trace_decay;
        presynapticFactor = p.presynaptic_factor;
        postsynapticFactor = p.postsynaptic_factor;
        seed = p.seed;
        if (n_neurons > 0) {
            int64_t s = 0;
            xyz_.resize(3 * (size_t)n_neurons);
            check(nc_reference_positions(n_neurons, xyz_.data()));
            check(nc_reference_connection_count(n_neurons, xyz_.data(), &s));
            from_.resize((size_t)s);
            to_.resize((size_t)s);
            w_.resize((size_t)s);
            check(nc_reference_connections(n_neurons, xyz_.data(), from_.data(), to_.data(), w_.data(), s));
        }
    }

    NeuCor(NeuCor&& o) noexcept { *this = std::move(o); }
    NeuCor& operator=(NeuCor&& o) noexcept
    {
        if (this != &o) {
            if (net_) nc_destroy(net_);
            runSpeed = o.runSpeed; runAll = o.runAll; learningRate = o.learningRate;
            presynapticTraceDecay = o.presynapticTraceDecay; postsynapticTraceDecay = o.postsynapticTraceDecay;
            presynapticFactor = o.presynapticFactor; postsynapticFactor = o.postsynapticFactor; seed = o.seed;
            xyz_ = std::move(o.xyz_); from_ = std::move(o.from_); to_ = std::move(o.to_); w_ = std::move(o.w_);
            groups_ = std::move(o.groups_);
            inputArray_ = o.inputArray_;
            inputRates_ = std::move(o.inputRates_);
            net_ = o.net_;
            o.net_ = nullptr;
            for (int k = 0; k < 4; ++k) pushed_[k] = o.pushed_[k];
        }
        return *this;
    }
    NeuCor(const NeuCor&) = delete;
    NeuCor& operator=(const NeuCor&) = delete;
    ~NeuCor()
    {
        if (net_) nc_destroy(net_);
    }

    // public members, as in src/NeuCor.h:68-73
    float runSpeed;
    bool runAll;
    float learningRate;
    float presynapticTraceDecay, postsynapticTraceDecay;
    float presynapticFactor, postsynapticFactor;
    uint64_t seed;   // key of the counter-based background and input draws

    // NeuCor::run (src/NeuCor.cpp:583-617): one step of runSpeed ms
    void run(int steps = 1)
    {
        materialize();
        push_rates();
        push_input_rates();
        check(nc_run(net_, steps));
    }

    // NeuCor::setInputRateArray (src/NeuCor.cpp:46-64).  The array stays borrowed: its
    // rates are read again before every run, as the reference does.
    void setInputRateArray(float inputs[], unsigned inputCount, coord3 inputPositions[] = nullptr,
                           float inputRadius[] = nullptr)
    {
        materialize();
        std::vector<float> xyz;
        if (inputPositions)
            for (unsigned i = 0; i < inputCount; ++i) {
                xyz.push_back(inputPositions[i].x);
                xyz.push_back(inputPositions[i].y);
                xyz.push_back(inputPositions[i].z);
            }
        check(nc_set_input_rate_array(net_, inputs, inputCount, inputPositions ? xyz.data() : nullptr, inputRadius));
        inputArray_ = inputs;
        inputRates_.assign(inputs, inputs + inputCount);
    }
    void addInputOffset(unsigned inputID, float t)        // src/NeuCor.cpp:66-68
    {
        materialize();
        check(nc_add_input_offset(net_, (int32_t)inputID, t));
    }
    void setDetectors(unsigned detectorNumber, coord3 detectorPositions[] = nullptr,
                      float detectorRadius[] = nullptr)  // src/NeuCor.cpp:70-77
    {
        materialize();
        std::vector<float> xyz;
        if (detectorPositions)
            for (unsigned i = 0; i < detectorNumber; ++i) {
                xyz.push_back(detectorPositions[i].x);
                xyz.push_back(detectorPositions[i].y);
                xyz.push_back(detectorPositions[i].z);
            }
        check(nc_set_detectors(net_, (int32_t)detectorNumber, detectorPositions ? xyz.data() : nullptr,
                               detectorRadius));
    }
    float getDetectorVoltage(unsigned ID)                  // src/NeuCor.cpp:75-77
    {
        materialize();
        float v = 0.0f;
        check(nc_get_detector_voltage(net_, (int32_t)ID, &v));
        return v;
    }
    std::vector<float> getDetectorVoltages()               // src/NeuCor.cpp:79-83
    {
        materialize();
        int32_t n = 0;
        check(nc_get_detector_voltages(net_, nullptr, 0, &n));
        std::vector<float> v((size_t)n);
        if (n) check(nc_get_detector_voltages(net_, v.data(), n, &n));
        return v;
    }
    float getTime() const
    {
        if (!net_) return 0.0f;
        float t = 0.0f;
        check(nc_get_time(net_, &t));
        return t;
    }

    void createNeuron(coord3 position)     // src/NeuCor.cpp:154
    {
        fixed();
        xyz_.push_back(position.x);
        xyz_.push_back(position.y);
        xyz_.push_back(position.z);
    }
    void createSynapse(std::size_t toID, std::size_t fromID, float weight)  // src/NeuCor.cpp:187
    {
        fixed();
        from_.push_back((int32_t)fromID);
        to_.push_back((int32_t)toID);
        w_.push_back(weight);
    }
    std::size_t getNeuronCount() const { return xyz_.size() / 3; }

    // Poisson input groups (see nc_group)
    void setInputGroups(const std::vector<nc_group>& groups)
    {
        groups_ = groups;
        if (net_) check(nc_set_input_groups(net_, (int32_t)groups_.size(), groups_.data()));
    }
    // Neuron::scheduleFire for the next step (src/NeuCor.cpp:658-661)
    void scheduleFire(const std::vector<int32_t>& ids)
    {
        materialize();
        check(nc_schedule_fire(net_, (int32_t)ids.size(), ids.data()));
    }

    std::vector<NeuronSnapshot> getNeuronSnapshots()      // src/NeuCor.cpp:99-113
    {
        materialize();
        const size_t n = getNeuronCount();
        std::vector<float> pa(2 * n);
        check(nc_read_potact(net_, pa.data()));
        std::vector<NeuronSnapshot> out(n);
        for (size_t i = 0; i < n; ++i)
            out[i] = NeuronSnapshot{i, coord3{xyz_[3 * i], xyz_[3 * i + 1], xyz_[3 * i + 2]}, pa[2 * i], pa[2 * i + 1]};
        return out;
    }
    struct InputSnapshot {        // src/NeuCor.h:56-62
        std::size_t id;
        coord3 position;
        float radius;
        float frequency;
        bool enabled;
    };
    std::vector<InputSnapshot> getInputSnapshots()       // src/NeuCor.cpp:136-152
    {
        materialize();
        push_rates();
        int32_t n = 0;
        check(nc_read_input_snapshots(net_, nullptr, 0, &n));
        std::vector<nc_input_snapshot> raw((size_t)n);
        if (n) check(nc_read_input_snapshots(net_, raw.data(), n, &n));
        std::vector<InputSnapshot> out;
        out.reserve(raw.size());
        for (const auto& r : raw)
            out.push_back(InputSnapshot{(std::size_t)r.id, coord3{r.x, r.y, r.z}, r.radius, r.frequency, r.enabled != 0});
        return out;
    }
    std::vector<SynapseSnapshot> getSynapseSnapshots()    // src/NeuCor.cpp:115-134
    {
        materialize();
        int64_t cnt = 0;
        check(nc_read_synapse_snapshots(net_, nullptr, 0, &cnt));
        std::vector<nc_synapse_snapshot> raw((size_t)cnt);
        check(nc_read_synapse_snapshots(net_, raw.data(), cnt, &cnt));
        std::vector<SynapseSnapshot> out;
        out.reserve((size_t)cnt);
        for (const auto& s : raw) {
            const size_t a = (size_t)s.from_id, b = (size_t)s.to_id;
            out.push_back(SynapseSnapshot{a, b, coord3{xyz_[3 * a], xyz_[3 * a + 1], xyz_[3 * a + 2]},
                                          coord3{xyz_[3 * b], xyz_[3 * b + 1], xyz_[3 * b + 2]}, s.weight,
                                          s.pre_potential, s.post_potential, s.inhibitory != 0});
        }
        return out;
    }
    // potAct (src/NeuCor.h:105)
    std::vector<float> potAct()
    {
        materialize();
        std::vector<float> pa(2 * getNeuronCount());
        check(nc_read_potact(net_, pa.data()));
        return pa;
    }
    // Synapse weights in creation order
    std::vector<float> weights()
    {
        materialize();
        std::vector<float> w(w_.size());
        check(nc_read_weights(net_, w.data()));
        return w;
    }
    void resetActivities()                                // src/NeuCor.cpp:233-235
    {
        materialize();
        check(nc_reset_activities(net_));
    }
    nc_net* handle()
    {
        materialize();
        return net_;
    }

private:
    void fixed() const
    {
        if (net_) throw Error(NC_ERR_UNSUPPORTED, "topology is fixed once the network is on the GPU");
    }
    void materialize()
    {
        if (net_) return;
        nc_params p;
        check(nc_default_params(&p));
        p.run_speed = runSpeed;
        p.learning_rate = learningRate;
        p.presynaptic_trace_decay = presynapticTraceDecay;
        p.postsynaptic_trace_decay = postsynapticTraceDecay;
        p.presynaptic_factor = presynapticFactor;
        p.postsynaptic_factor = postsynapticFactor;
        p.seed = seed;
        check(nc_create((int32_t)getNeuronCount(), xyz_.data(), (int64_t)w_.size(), from_.data(), to_.data(),
                        w_.data(), nullptr, nullptr, &p, &net_));
        if (!groups_.empty()) check(nc_set_input_groups(net_, (int32_t)groups_.size(), groups_.data()));
        pushed_[0] = learningRate;
        pushed_[1] = presynapticFactor;
        pushed_[2] = postsynapticFactor;
        pushed_[3] = runSpeed;
    }
    void push_rates()
    {
        if (runSpeed != pushed_[3]) throw Error(NC_ERR_UNSUPPORTED, "runSpeed is fixed once the network is on the GPU");
        if (learningRate != pushed_[0] || presynapticFactor != pushed_[1] || postsynapticFactor != pushed_[2]) {
            check(nc_set_rates(net_, learningRate, presynapticFactor, postsynapticFactor));
            pushed_[0] = learningRate;
            pushed_[1] = presynapticFactor;
            pushed_[2] = postsynapticFactor;
        }
    }

    std::vector<float> xyz_;
    std::vector<int32_t> from_, to_;
    std::vector<float> w_;
    void push_input_rates()
    {
        if (!inputArray_) return;
        bool changed = false;
        for (size_t i = 0; i < inputRates_.size(); ++i) changed |= inputRates_[i] != inputArray_[i];
        if (!changed) return;
        inputRates_.assign(inputArray_, inputArray_ + inputRates_.size());
        check(nc_set_input_rates(net_, (int32_t)inputRates_.size(), inputRates_.data()));
    }

    std::vector<nc_group> groups_;
    const float* inputArray_ = nullptr;  // borrowed, as NeuCor::inputArray
    std::vector<float> inputRates_;      // the rates last pushed
    nc_net* net_ = nullptr;
    float pushed_[4] = {0, 0, 0, 0};
};

}  // namespace neucor_gb300
#endif
