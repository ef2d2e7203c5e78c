// Oracle-R harness — drives the reference's own simulator core (src/NeuCor.cpp,
// compiled unmodified from the reference tree by oracle/Makefile) on a scenario
// file and writes what it computed.  TEST INFRASTRUCTURE: used here to pin the
// stepped restatement (nc_oracle.c) and to make the golden fixtures.
//
// Access to the simulator's internals goes through the reference's own friend
// hook: `friend class NeuCor_Renderer` (NeuCor.h:98, NeuCor.h:270), which the
// reference gives its renderer.  This file defines a class of that name.
//
// The reference calls the C library's rand() for construction, background
// firing and a dead branch of the plasticity rule (NeuCor.cpp:12-14, 471-473,
// 606, 752).  The Makefile links with `ld --wrap=rand`, so those calls reach
// __wrap_rand below, and background firing can be driven from the same
// counter-based draws as the stepped model.
//
// Modes:
//   0 canonical  — the reference's Neuron/Synapse code, run by a stepped
//                  scheduler: all neurons in ascending id at each T
//                  (Neuron::run, NeuCor.cpp:619), then the queued events of T
//                  (Synapse::run, NeuCor.cpp:718) in the reference's heap.
//   1 native     — the reference's own NeuCor::run (NeuCor.cpp:583-617) with
//                  runAll=true, runSpeed=dt; the harness then runs every neuron
//                  at the new T so each step ends with all neurons updated.
//   2 continuous — NeuCor::run alone, synapse lengths as constructed (spikes
//                  arrive between steps), background firing from glibc rand().
//   3 continuous on the step grid — as 2, with every synapse length set to its
//                  whole-step delay (separates the effect of delay rounding from
//                  that of the off-grid background fire times).
//   4 construct  — srand(seed); NeuCor(n) (NeuCor.cpp:17-42); writes the positions
//                  and every synapse (source, target, weight, length) in the
//                  reference's own order.
//   5 inputs     — srand(seed); NeuCor(0) with the scenario's neurons; then
//                  setInputRateArray(rates, count, NULL, NULL) (random firer
//                  positions, NeuCor.cpp:46-64, 309-313); writes getInputSnapshots.
// Modes 0, 1 and 3 set every synapse length to delay*dt/AP_speed so spikes arrive
// on the step grid.
#include "NeuCor.h"
#include "nc_oracle.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <utility>
#include <vector>

// ------------------------------------------------------------------ rand()
namespace {
int g_rand_mode = 0;  // 0: glibc rand; 1: background loop; 2: after it
const uint8_t* g_hit = nullptr;
const int32_t* g_target = nullptr;
int32_t g_n = 0, g_i = 0, g_sub = 0;
}  // namespace

extern "C" int __real_rand(void);

extern "C" int __wrap_rand(void)
{
    if (g_rand_mode == 1) {
        // NeuCor.cpp:605-606: `if (rand()%period == 0) neurons.at(rand()%N).scheduleFire(randomUnit()*runSpeed)`
        if (g_i >= g_n) { g_rand_mode = 2; return 1; }
        if (g_sub == 0) {
            if (g_hit[g_i]) { g_sub = 1; return 0; }
            if (++g_i == g_n) g_rand_mode = 2;
            return 1;
        }
        if (g_sub == 1) { g_sub = 2; return g_target[g_i]; }
        g_sub = 0;
        if (++g_i == g_n) g_rand_mode = 2;
        return RAND_MAX;  // randomUnit() == 1.0f: the fire lands on the next step
    }
    if (g_rand_mode == 2) return 1;  // only NeuCor.cpp:752, whose condition ends in `&& false`
    return __real_rand();
}

// ---------------------------------------------------------------- scenario
struct Scenario {
    int32_t mode = 0, n = 0;
    int64_t s = 0;
    std::vector<float> xyz;
    std::vector<int32_t> pre, post;
    std::vector<float> w;
    ncs_params p{};
    std::vector<ncs_group> groups;
    int32_t steps = 0, record_pot = 0;
    std::vector<std::pair<int32_t, int32_t>> extra;  // (step, id): forced fire requests
    std::vector<int32_t> checkpoints;
    // periodic input firers (NeuCor::setInputRateArray, NeuCor.cpp:46-64), continuous mode only
    std::vector<coord3> firer_pos;
    std::vector<float> firer_radius, firer_rate, firer_offset;
    // voltage detectors (NeuCor::setDetectors, NeuCor.cpp:70-77): position and radius
    std::vector<coord3> det_pos;
    std::vector<float> det_radius;
};

template <class T>
static void rd(FILE* f, T* v, size_t n = 1)
{
    if (n && fread(v, sizeof(T), n, f) != n) { fprintf(stderr, "short scenario file\n"); exit(2); }
}

static Scenario read_scenario(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) { perror(path); exit(2); }
    Scenario sc;
    char magic[4];
    rd(f, magic, 4);
    if (memcmp(magic, "NCRF", 4) != 0) { fprintf(stderr, "bad magic\n"); exit(2); }
    rd(f, &sc.mode); rd(f, &sc.n); rd(f, &sc.s);
    sc.xyz.resize(3 * (size_t)sc.n); rd(f, sc.xyz.data(), sc.xyz.size());
    sc.pre.resize(sc.s); sc.post.resize(sc.s); sc.w.resize(sc.s);
    rd(f, sc.pre.data(), sc.s); rd(f, sc.post.data(), sc.s); rd(f, sc.w.data(), sc.s);
    float fp[6]; rd(f, fp, 6);
    sc.p.run_speed = fp[0]; sc.p.learning_rate = fp[1];
    sc.p.presynaptic_trace_decay = fp[2]; sc.p.postsynaptic_trace_decay = fp[3];
    sc.p.presynaptic_factor = fp[4]; sc.p.postsynaptic_factor = fp[5];
    rd(f, &sc.p.background_firing); rd(f, &sc.p.seed);
    int32_t ng; rd(f, &ng); sc.groups.resize(ng);
    for (auto& g : sc.groups) { rd(f, &g.first); rd(f, &g.count); rd(f, &g.rate_hz); rd(f, &g.correlated); rd(f, &g.jitter); }
    rd(f, &sc.steps); rd(f, &sc.record_pot);
    int32_t ne; rd(f, &ne); sc.extra.resize(ne);
    for (auto& e : sc.extra) { rd(f, &e.first); rd(f, &e.second); }
    int32_t nc; rd(f, &nc); sc.checkpoints.resize(nc); rd(f, sc.checkpoints.data(), nc);
    int32_t nf; rd(f, &nf);
    for (int32_t i = 0; i < nf; ++i) {
        float v[6]; rd(f, v, 6);
        sc.firer_pos.push_back(coord3{v[0], v[1], v[2]});
        sc.firer_radius.push_back(v[3]); sc.firer_rate.push_back(v[4]); sc.firer_offset.push_back(v[5]);
    }
    int32_t nd = 0;
    if (fread(&nd, sizeof(nd), 1, f) != 1) nd = 0;  // older scenario files end here
    for (int32_t i = 0; i < nd; ++i) {
        float v[4]; rd(f, v, 4);
        sc.det_pos.push_back(coord3{v[0], v[1], v[2]});
        sc.det_radius.push_back(v[3]);
    }
    fclose(f);
    return sc;
}

// ------------------------------------------------------------------ harness
class NeuCor_Renderer;
struct NeuCor_Lengths {
    static void collect(NeuCor& brain, std::vector<float>& out);
};

class NeuCor_Renderer {
public:
    explicit NeuCor_Renderer(const Scenario& sc) : sc_(sc) {}

    int run(const char* out_path)
    {
        const int32_t n = sc_.n;
        const float dt = sc_.p.run_speed;
        brain_ = new NeuCor(0);
        // Decays are copied into each Neuron/Synapse at construction (NeuCor.cpp:369,464).
        brain_->presynapticTraceDecay = sc_.p.presynaptic_trace_decay;
        brain_->postsynapticTraceDecay = sc_.p.postsynaptic_trace_decay;
        brain_->presynapticFactor = sc_.p.presynaptic_factor;
        brain_->postsynapticFactor = sc_.p.postsynaptic_factor;
        brain_->learningRate = sc_.p.learning_rate;
        brain_->runSpeed = dt;
        brain_->runAll = true;
        for (int32_t i = 0; i < n; ++i)
            brain_->createNeuron(coord3{sc_.xyz[3 * i], sc_.xyz[3 * i + 1], sc_.xyz[3 * i + 2]});
        std::set<std::pair<int32_t, int32_t>> seen;
        first_.assign(sc_.s, 0);
        for (int64_t k = 0; k < sc_.s; ++k) {
            first_[k] = seen.insert({sc_.pre[k], sc_.post[k]}).second;
            brain_->createSynapse(sc_.post[k], sc_.pre[k], sc_.w[k]);
        }
        if (sc_.mode != 2) {
            for (auto& neu : brain_->neurons)
                for (auto& syn : neu.outSynapses) syn.length = (float)ncs_delay_steps(syn.length, dt) * dt / syn.AP_speed;
        }
        if (!sc_.firer_rate.empty()) {
            rates_ = sc_.firer_rate;  // the brain keeps this pointer and re-reads it every run()
            brain_->setInputRateArray(rates_.data(), (unsigned)rates_.size(),
                                      const_cast<coord3*>(sc_.firer_pos.data()),
                                      const_cast<float*>(sc_.firer_radius.data()));
            for (size_t i = 0; i < rates_.size(); ++i)
                if (sc_.firer_offset[i] != 0.0f) brain_->addInputOffset((unsigned)i, sc_.firer_offset[i]);
        }
        if (!sc_.det_radius.empty())
            brain_->setDetectors((unsigned)sc_.det_radius.size(), const_cast<coord3*>(sc_.det_pos.data()),
                                 const_cast<float*>(sc_.det_radius.data()));
        // scheduledFireTime is never initialised by the Neuron constructor
        // (NeuCor.cpp:368-395); give it a time that is never reached.
        for (auto& neu : brain_->neurons) neu.scheduleFire(1e30f);

        FILE* out = fopen(out_path, "wb");
        if (!out) { perror(out_path); return 2; }
        const size_t row = ((size_t)n + 7) / 8;
        std::vector<uint8_t> raster(row * (size_t)sc_.steps, 0);
        std::vector<float> pots;
        if (sc_.record_pot) pots.resize((size_t)n * sc_.steps);
        std::vector<float> ckw;
        std::vector<uint8_t> cks;   // synapse snapshots at the checkpoints (packed records)
        std::vector<float> volts;   // detector voltages at the checkpoints
        std::vector<float> firer_last;  // InputFirer::lastFire of every firer after each run call
        std::vector<uint8_t> hit(n);
        std::vector<int32_t> target(n), ids(n > 0 ? n : 1);
        size_t ck = 0;

        if (sc_.mode == 0) {
            // step 0: neuron runs at T=0 return at once; draws and requests for step 1
            schedule_step_requests(1, dt, hit, target, ids);
        }
        for (int32_t t = 1; t <= sc_.steps; ++t) {
            if (sc_.mode == 0) {
                brain_->currentTime = brain_->currentTime + dt;
                const float T = brain_->currentTime;
                for (auto& neu : brain_->neurons) neu.run();
                auto& q = brain_->simulationQueue;
                while (!q.empty() && q.top().stime <= T) {
                    q.top().addr->run();
                    q.pop();
                }
                if (t < sc_.steps) schedule_step_requests(t + 1, dt, hit, target, ids);
            } else {
                request_inputs(t, dt, ids);
                if (sc_.mode == 1 && sc_.p.background_firing) {
                    ncs_background_draws(sc_.p.seed, n, dt, t - 1, hit.data(), target.data());
                    g_hit = hit.data(); g_target = target.data(); g_n = n; g_i = 0; g_sub = 0;
                    g_rand_mode = 1;
                } else if (sc_.mode == 1) {
                    // background loop still runs; make every draw miss
                    std::fill(hit.begin(), hit.end(), 0);
                    g_hit = hit.data(); g_target = target.data(); g_n = n; g_i = 0; g_sub = 0;
                    g_rand_mode = 1;
                } else {
                    g_rand_mode = 0;
                }
                brain_->run();
                if (sc_.mode == 1) {
                    g_rand_mode = 2;
                    for (auto& neu : brain_->neurons) neu.run();
                }
            }
            for (auto& firer : brain_->inputHandler) firer_last.push_back(firer.lastFire);
            const float T = brain_->currentTime;
            uint8_t* rr = &raster[row * (size_t)(t - 1)];
            for (int32_t j = 0; j < n; ++j) {
                const float lf = brain_->neurons[j].lastFire;
                bool fired = (sc_.mode == 2 || sc_.mode == 3) ? (lf == lf && lf > T - dt && lf <= T) : (lf == T);
                if (fired) rr[j >> 3] |= (uint8_t)(1u << (j & 7));
                if (sc_.record_pot) pots[(size_t)(t - 1) * n + j] = brain_->potAct[2 * (size_t)j];
            }
            while (ck < sc_.checkpoints.size() && sc_.checkpoints[ck] == t) {
                append_weights(ckw);
                append_snapshots(cks);
                for (float v : brain_->getDetectorVoltages()) volts.push_back(v);
                ck++;
            }
        }
        fwrite(raster.data(), 1, raster.size(), out);
        if (sc_.record_pot) fwrite(pots.data(), sizeof(float), pots.size(), out);
        fwrite(ckw.data(), sizeof(float), ckw.size(), out);
        std::vector<float> fin(3 * (size_t)n);
        for (int32_t j = 0; j < n; ++j) {
            fin[j] = brain_->potAct[2 * (size_t)j];
            fin[n + j] = brain_->potAct[2 * (size_t)j + 1];
            fin[2 * n + j] = brain_->neurons[j].lastFire;
        }
        fwrite(fin.data(), sizeof(float), fin.size(), out);
        // the reference's own Synapse::inhibitory flags (never changed after construction)
        std::vector<uint8_t> inh(sc_.s, 255);
        for (int64_t k = 0; k < sc_.s; ++k) {
            if (!first_[k]) continue;
            const Synapse* syn = brain_->getSynapse((std::size_t)sc_.pre[k], (std::size_t)sc_.post[k]);
            inh[k] = syn && syn->inhibitory ? 1 : 0;
        }
        fwrite(inh.data(), 1, inh.size(), out);
        fwrite(firer_last.data(), sizeof(float), firer_last.size(), out);
        // NeuCor::getSynapseSnapshots at every checkpoint, then getDetectorVoltages
        fwrite(cks.data(), 1, cks.size(), out);
        fwrite(volts.data(), sizeof(float), volts.size(), out);
        fclose(out);
        delete brain_;
        return 0;
    }

private:
    void request_inputs(int32_t t, float dt, std::vector<int32_t>& ids)
    {
        // Requests for step t, made while the brain is at step t-1:
        // Neuron::scheduleFire(dt) sets scheduledFireTime = T (NeuCor.cpp:658-661).
        int32_t cnt = ncs_input_fires(sc_.groups.data(), (int32_t)sc_.groups.size(), sc_.p.seed, dt, t,
                                      ids.data(), (int32_t)ids.size());
        for (int32_t k = 0; k < cnt && k < (int32_t)ids.size(); ++k) brain_->neurons[ids[k]].scheduleFire(dt);
        for (auto& e : sc_.extra)
            if (e.first == t) brain_->neurons[e.second].scheduleFire(dt);
    }

    void schedule_step_requests(int32_t t, float dt, std::vector<uint8_t>& hit, std::vector<int32_t>& target,
                                std::vector<int32_t>& ids)
    {
        const int32_t n = sc_.n;
        if (sc_.p.background_firing && n > 0) {
            ncs_background_draws(sc_.p.seed, n, dt, t - 1, hit.data(), target.data());
            for (int32_t i = 0; i < n; ++i)
                if (hit[i]) brain_->neurons[target[i]].scheduleFire(dt);
        }
        request_inputs(t, dt, ids);
    }

    // Per checkpoint: int64 count, then count records of {int32 from, int32 to, float
    // weight, float prePotential, float postPotential, uint8 inhibitory} (21 bytes).
    void append_snapshots(std::vector<uint8_t>& out)
    {
        const auto snaps = brain_->getSynapseSnapshots();
        const int64_t c = (int64_t)snaps.size();
        const uint8_t* cp = (const uint8_t*)&c;
        out.insert(out.end(), cp, cp + sizeof(c));
        for (const auto& sn : snaps) {
            const int32_t ids[2] = {(int32_t)sn.fromID, (int32_t)sn.toID};
            const float v[3] = {sn.weight, sn.prePotential, sn.postPotential};
            const uint8_t* a = (const uint8_t*)ids;
            out.insert(out.end(), a, a + sizeof(ids));
            const uint8_t* b = (const uint8_t*)v;
            out.insert(out.end(), b, b + sizeof(v));
            out.push_back(sn.inhibitory ? 1 : 0);
        }
    }

    void append_weights(std::vector<float>& out)
    {
        for (int64_t k = 0; k < sc_.s; ++k) {
            if (!first_[k]) { out.push_back(NAN); continue; }
            const Synapse* syn = brain_->getSynapse((std::size_t)sc_.pre[k], (std::size_t)sc_.post[k]);
            out.push_back(syn ? syn->getWeight() : NAN);
        }
    }

    friend struct NeuCor_Lengths;
    static void lengths(NeuCor& brain, std::vector<float>& out)
    {
        for (auto& neu : brain.neurons)
            for (auto& syn : neu.outSynapses) out.push_back(syn.length);
    }

    const Scenario& sc_;
    NeuCor* brain_ = nullptr;
    std::vector<uint8_t> first_;
    std::vector<float> rates_;
};

void NeuCor_Lengths::collect(NeuCor& brain, std::vector<float>& out) { NeuCor_Renderer::lengths(brain, out); }

static int construct(const Scenario& sc, const char* out_path)
{
    srand((unsigned)sc.p.seed);
    NeuCor brain(sc.n);
    FILE* out = fopen(out_path, "wb");
    if (!out) { perror(out_path); return 2; }
    std::vector<float> xyz;
    std::vector<int32_t> from, to;
    std::vector<float> w, len;
    for (const auto& p : brain.getNeuronSnapshots()) { xyz.push_back(p.position.x); xyz.push_back(p.position.y); xyz.push_back(p.position.z); }
    for (const auto& s : brain.getSynapseSnapshots()) { from.push_back((int32_t)s.fromID); to.push_back((int32_t)s.toID); w.push_back(s.weight); }
    NeuCor_Lengths::collect(brain, len);
    int64_t ns = (int64_t)from.size();
    fwrite(&ns, sizeof(ns), 1, out);
    fwrite(xyz.data(), sizeof(float), xyz.size(), out);
    fwrite(from.data(), sizeof(int32_t), from.size(), out);
    fwrite(to.data(), sizeof(int32_t), to.size(), out);
    fwrite(w.data(), sizeof(float), w.size(), out);
    fwrite(len.data(), sizeof(float), len.size(), out);
    fclose(out);
    return 0;
}

static int inputs(const Scenario& sc, const char* out_path)
{
    srand((unsigned)sc.p.seed);
    NeuCor brain(0);
    for (int32_t i = 0; i < sc.n; ++i) brain.createNeuron(coord3{sc.xyz[3 * i], sc.xyz[3 * i + 1], sc.xyz[3 * i + 2]});
    std::vector<float> rates = sc.firer_rate;  // borrowed by the brain, as in NeuCor
    brain.setInputRateArray(rates.data(), (unsigned)rates.size(), nullptr, nullptr);
    FILE* out = fopen(out_path, "wb");
    if (!out) { perror(out_path); return 2; }
    for (const auto& s : brain.getInputSnapshots()) {
        const float v[6] = {(float)s.id, s.position.x, s.position.y, s.position.z, s.radius, s.frequency};
        fwrite(v, sizeof(float), 6, out);
        const uint8_t en = s.enabled ? 1 : 0;
        fwrite(&en, 1, 1, out);
    }
    fclose(out);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s scenario.bin out.bin\n", argv[0]);
        return 2;
    }
    Scenario sc = read_scenario(argv[1]);
    if (sc.mode == 4) return construct(sc, argv[2]);
    if (sc.mode == 5) return inputs(sc, argv[2]);
    srand((unsigned)sc.p.seed);
    NeuCor_Renderer drv(sc);
    return drv.run(argv[2]);
}
