// CPU oracle for the GB300 PIC deposition path -- TEST INFRASTRUCTURE ONLY
// (see pic_oracle.h for who may call it).
//
// sortParticlesByCell(ParticlesSoA&, const Domain&) (src/sorting/cell_sort.cpp:22-46)
// restated over six FP64 arrays: an index array sorted with std::sort by
// particleCellIndex (cell_sort.cpp:8-13), the key computed for both operands of
// every comparison as the reference's comparator does, then each array gathered
// through the order. std::sort is not stable; with the same keys and the same
// standard library the order equals the reference's.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "pic_oracle.h"

extern "C" int orc_sort_particles_by_cell(const orc_domain* d, size_t n, double* x, double* y, double* vx, double* vy,
                                          double* q, double* m) {
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return orc_particle_cell_index(d, x[a], y[a]) < orc_particle_cell_index(d, x[b], y[b]);
    });
    std::vector<double> tmp(n);
    double* arrays[6] = {x, y, vx, vy, q, m};
    for (double* a : arrays) {
        for (size_t i = 0; i < n; ++i) tmp[i] = a[order[i]];
        std::memcpy(a, tmp.data(), n * sizeof(double));
    }
    return 0;
}
