// och_gel.cpp — initial gel order parameter of the CPU oracle (test
// infrastructure only).
//
// src/mobility/GelMobility.h:28-33 of the reference draws it once, at
// construction, from a default-seeded std::mt19937 through
// std::uniform_real_distribution<double>(0, 1), times 1e-4.  The C++ standard
// library fixes the engine; the distribution is the toolchain's (libstdc++
// here, as for the reference's own build), so the oracle calls it the same way.
#include <cstddef>
#include <random>

extern "C" void och_gel_init(double *op, size_t n) {
    std::mt19937 generator;
    std::uniform_real_distribution<double> dist(0.0, 1.0);
    for(size_t i = 0; i < n; i++) op[i] = dist(generator) * 1e-4;
}
