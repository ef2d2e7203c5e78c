// The reference's FEW_NEURONS preset (src/main.cpp:162-189) written against the
// reference's class interface, built on include/neucor_gb300.hpp: three neurons,
// synapses 0->1 and 0->2 at 0.5, each neuron driven every 20 ms (neuron 1 two
// steps later, neuron 2 two steps earlier).  Prints the two weights at 50/100/150/250 ms.
#include <cstdio>
#include <vector>

#include "neucor_gb300.hpp"

int main()
{
    using neucor_gb300::NeuCor;
    NeuCor brain(0);
    brain.runAll = true;
    brain.runSpeed = 1.0f;
    brain.seed = 1;
    brain.createNeuron({0.0f, 0.0f, 0.0f});
    brain.createNeuron({0.3f, 0.3f, 0.0f});
    brain.createNeuron({0.3f, -0.3f, 0.0f});
    brain.createSynapse(1, 0, 0.5f);
    brain.createSynapse(2, 0, 0.5f);
    const int offsets[3] = {0, 2, -2};
    for (int t = 1; t <= 250; ++t) {
        std::vector<int32_t> due;
        for (int i = 0; i < 3; ++i)
            if ((t - offsets[i]) % 20 == 0 && t - offsets[i] > 0) due.push_back(i);
        if (!due.empty()) brain.scheduleFire(due);
        brain.run();
        if (t == 50 || t == 100 || t == 150 || t == 250) {
            std::vector<float> w = brain.weights();
            std::printf("%d %.9g %.9g\n", t, w[0], w[1]);
        }
    }
    std::printf("time %.3f neurons %zu synapses %zu\n", brain.getTime(), brain.getNeuronCount(),
                brain.getSynapseSnapshots().size());
    return 0;
}
