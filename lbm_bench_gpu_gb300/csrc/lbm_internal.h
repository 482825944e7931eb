// lbm_internal.h -- shared definitions of liblbm_gb300 (not part of the C-ABI).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>

#include "lbm_gb300.h"

namespace lbm {

// D3Q7 (f) and D3Q19 (g) lattice vectors in the reference order
// (src/stream_f.cu:52-59, src/stream_g.cu:122-142).
// f: 0 rest, 1 +x, 2 -x, 3 +y, 4 -y, 5 +z, 6 -z
// g: 0 rest, 1..6 as f, 7 (+x+y), 8 (-x-y), 9 (+x-y), 10 (-x+y), 11 (+x+z),
//    12 (-x-z), 13 (+x-z), 14 (-x+z), 15 (+y+z), 16 (-y-z), 17 (+y-z), 18 (-y+z)
constexpr int kQf = 7;
constexpr int kQg = 19;

// Scalars the step needs, all FP32 (src/constants.h:81-85 plus grav_d).
struct StepConst {
    float eta, eta2;                          // ZSC streaming interpolation
    float alpha4, kappa, phiStarSq, Gamma;    // chemical potential
    float invTauPhi, invTauPhiOne, invEta2;   // D3Q7 relaxation
    float invTauRhoOne, K0, K1, K2, KC0, KC1, KC2;  // D3Q19 relaxation + forcing
    float grav;                               // body force on phi > 0 nodes
};

// Box of interior nodes, periodic in x, y, z.
struct Box {
    int nx, ny, nz;
    long long nxy, n;
};

// Device buffers of one context.
//  f      : 2 x 7 x n   post-collision D3Q7 values (A/B by step parity), or the
//           streamed initial values while `f_streamed` is set
//  g      : 19 x n      D3Q19 values in the in-place AA layout
//  mom    : 5 x n       phi, rho, ux, uy, uz as the reference's arrays hold them
struct State {
    float *f = nullptr;
    float *g = nullptr;
    float *mom = nullptr;
    int f_cur = 0;            // which half of f holds the current values
    bool f_streamed = true;   // f holds streamed (not post-collision) values
    long long steps = 0;      // steps since init; AA parity = steps & 1
};

// Scratch for reductions (per-block partials), owned by the context.
struct Scratch {
    double *partials = nullptr;
    size_t partial_count = 0;
    double *result = nullptr;      // final reduced values
    unsigned long long *counters = nullptr;
};

void set_error(const std::string &msg);
const std::string &last_error();

// Host-side derivation of the constants (src/paramread.c:141-170).
void derive(const lbm_params &p, lbm_derived &d);
StepConst step_const(const lbm_derived &d, const lbm_params &p, float grav);

// Kernel launchers (defined in the .cu files); all return cudaError_t of the launch.
cudaError_t launch_bubble_phi(const Box &b, const float *bubbles_dev, int nbubbles, float phiStar, float width,
                              float *phi_ghosted, cudaStream_t s);
cudaError_t launch_equilibrium(const Box &b, const lbm_derived &d, float Gamma, const float *phi, const float *rho,
                               const float *ghost_lo, const float *ghost_hi, float *f, float *g, cudaStream_t s);
cudaError_t launch_fill(float *p, long long n, float v, cudaStream_t s);
cudaError_t launch_step(const Box &b, const StepConst &c, const float *f_in, float *f_out, float *g, float *mom,
                        bool f_streamed, bool odd, bool write_moments, cudaStream_t s);
cudaError_t launch_stream_out(const Box &b, float eta, const float *f_state, bool f_streamed, const float *g,
                              bool odd, float *f_out, float *g_out, cudaStream_t s);
cudaError_t launch_moments(const Box &b, const float *f, const float *g, float *mom, cudaStream_t s);
cudaError_t launch_stats(const Box &b, const lbm_derived &d, const float *mom, double *partials,
                         size_t partial_count, double *result, unsigned long long *counters, cudaStream_t s);
size_t stats_partial_count(const Box &b);

// Number of doubles produced by launch_stats in `result`.
constexpr int kStatsValues = 16;

}  // namespace lbm
