// Data types of the batched form shared by its host code (batch.cu,
// serve.cu) and its kernels (batch_kernels.cuh).
#pragma once

#include <cstddef>

namespace dg {

constexpr int BATCH_THREADS = 256;
constexpr int BATCH_KMAX = 6;

struct BatchProblem {
    int K, np, n_elem, src_face;
    int active, cur, steps_left, pad;
    float* u[2];           // ping-pong state, 4 fields each
    float* comp;           // Kahan compensation
    float* d[2];           // stage increments d1, d2
    float* q;              // LDG gradient times -D_c, 3 fields
    const int* nbr;        // n_elem x 6, problem-local; boundary: -1 - face
    const float* sigma;    // n_elem
    size_t fs;             // field stride n_elem * np
    // rows[i] = (D[i][0..K-1], L0[i], LN[i], 0...): the unit-interval
    // derivative row and the lift entries of node i, 16-byte aligned so a
    // thread loads its row with two vector loads.
    alignas(16) float rows[BATCH_KMAX][8];
    float invw[3];         // 1 / w_a
    float gscale[3];       // D_c / w_a
    float cM[2][4], cA[2][4];  // face coefficients with the lift scales, w factored out
    float k1, k2, r0, inv_c2, inv_z;
    int linear_mass;
    float ca[3], cb[3], eps;   // R weight, increment weight, u weight of each stage
    float src_p[3];        // source pressure at the three stage times of this step
    double t, dt;
    double src_amp, src_freq, src_T, src_phase;
    long long steps_done;
};

// The unit-interval operator rows of one order (same layout as
// BatchProblem::rows), passed by value to the kernel of a group of problems
// that share them, so that the line owners read constant-bank operands.
struct BatchOps {
    float rows[BATCH_KMAX][8];
};

struct BatchTile {
    int prob, e0, count, K;
};

struct BatchArgs {
    BatchProblem* probs;
    const BatchTile* tiles;
    int tile0, n_tiles;    // this launch's tiles: tiles[tile0 .. tile0 + n_tiles)
    int* counters;         // [2]: phase-1 and phase-2 tile counters, zeroed before the launch
    int stage;
};

}  // namespace dg
