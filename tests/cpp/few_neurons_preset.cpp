// The reference's FEW_NEURONS preset as its own code sets it up (src/main.cpp:162-189):
// runSpeed 0.02 ms, three neurons, synapses 0->1 and 0->2 at 0.5, a 50 Hz periodic input
// on each neuron (radius 0.1) with the second shifted by +2 ms and the third by -2 ms —
// written against the reference's class interface, built on include/neucor_gb300.hpp.
// Prints the two weights at 50/100/150/250 ms of simulated time.
#include <cstdio>
#include <vector>

#include "neucor_gb300.hpp"

int main()
{
    using neucor_gb300::NeuCor;
    using neucor_gb300::coord3;
    NeuCor brain(0);
    brain.runAll = true;
    brain.runSpeed = 0.02f;
    brain.seed = 1;
    const std::vector<coord3> positions = {{0, 0, 0}, {0.3f, 0.3f, 0}, {0.3f, -0.3f, 0}};
    for (const coord3& p : positions) brain.createNeuron(p);
    brain.createSynapse(1, 0, 0.5f);
    brain.createSynapse(2, 0, 0.5f);
    std::vector<float> inputs = {50.0f, 50.0f, 50.0f};
    std::vector<coord3> input_positions(positions);
    std::vector<float> input_radius = {0.1f, 0.1f, 0.1f};
    brain.setInputRateArray(inputs.data(), (unsigned)inputs.size(), input_positions.data(), input_radius.data());
    brain.addInputOffset(1, 2.0f);
    brain.addInputOffset(2, -2.0f);
    const int marks[4] = {2500, 5000, 7500, 12500};  // 50, 100, 150, 250 ms at 0.02 ms per step
    int done = 0;
    for (int m = 0; m < 4; ++m) {
        brain.run(marks[m] - done);
        done = marks[m];
        std::vector<float> w = brain.weights();
        std::printf("%d %.9g %.9g\n", done, w[0], w[1]);
    }
    std::printf("time %.3f\n", brain.getTime());
    return 0;
}
