// Internal interface of the learned preconditioner network (mpm_nn.cu).
//
// The network is a 3-level convolutional encoder-decoder over the nodal grid
// (control points), channels-last BF16 activations, FP32 accumulation:
//
//   x0 = [r_u, r_v, r_w, phi_u, phi_v, phi_w, 0 x 10]  level 0 (n0 nodes), 16 ch
//   e0 = relu(conv3(x0; 6->16))                       level 0
//   e1 = relu(conv3/2(e0; 16->32))                    level 1 (n1 = n0/2 + 1)
//   e2 = relu(conv3/2(e1; 32->64))                    level 2 (n2 = n1/2 + 1)
//   c2 = conv3(e2; 64->32)                            level 2
//   d1 = relu(up(c2) + e1)                            level 1
//   c1 = conv3(d1; 32->16)                            level 1
//   d0 = relu(up(c1) + e0)                            level 0
//   z  = d0 W5 + b5 (16 -> 3)                         level 0, FP32
//
// conv3 is a 3x3x3 convolution with zero padding, conv3/2 the same with
// stride 2 (coarse node I sits on fine node 2I), up the node-aligned
// trilinear prolongation.  The five 3x3x3 convolutions (and their
// data-gradient and weight-gradient counterparts) run on tcgen05 tensor
// cores; the prolongation, restriction, 1x1 output layer and reductions on
// CUDA cores.  phi_c = (mass term of the diagonal entry) / (diagonal entry)
// of each degree of freedom tells the network how stiff the system is
// relative to its inertia (it is 1 for a mass-dominated row and small for a
// stiffness-dominated one), which the residual alone does not.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_gpu.h"

namespace mpm {
namespace nn {

constexpr int NCONV = 5;
constexpr int NIN = 6;   // input channels: residual (3) and the system's mass fractions (3)
constexpr int CIN[NCONV] = {NIN, 16, 32, 64, 32};
constexpr int COUT[NCONV] = {16, 32, 64, 32, 16};
constexpr int KPAD[NCONV] = {16, 16, 32, 64, 32};   // input channels as stored (x0 padded to 16)

int64_t param_count();
// offsets into the FP32 parameter vector: W_l [27][cin][cout], b_l [cout], W5 [16][3], b5 [3]
int64_t w_offset(int l);
int64_t b_offset(int l);
int64_t w5_offset();
int64_t b5_offset();

}  // namespace nn
}  // namespace mpm

// Preconditioner application for the implicit solver: z = s * net(r / s)
// with s = sqrt(rr / (3 nodec)) read from the device scalar rr; r and z are
// FP64, component-major (3 x nodec) in the diagonally scaled system, z is
// zeroed on inactive (adiag < mtol) and boundary-condition rows.
mpm_status mpm_nn_apply_precond(mpm_nn *net, cudaStream_t st, const double *r, const double *rr, const double *adiag,
                                const unsigned char *bcflag, double mtol, double *z);
// The same with z in FP32, for the network's default mode (linear, not
// symmetrised: true from mpm_nn_fp32_output); MPM_ERR_UNSUPPORTED otherwise.
mpm_status mpm_nn_apply_precond_f32(mpm_nn *net, cudaStream_t st, const double *r, const double *rr,
                                    const double *adiag, const unsigned char *bcflag, double mtol, float *z);
int mpm_nn_fp32_output(const mpm_nn *net);
// Feature channels of the system about to be solved (phi, FP64 component-major).
mpm_status mpm_nn_set_feature(mpm_nn *net, cudaStream_t st, const double *phi);
// Harvest: the features of a new system; the pairs appended next belong to it.
mpm_status mpm_nn_begin_system(mpm_nn *net, cudaStream_t st, const double *phi);
// Appends one (residual, error) pair, both scaled by the residual's RMS,
// to the training set (ignored once the set is full).
mpm_status mpm_nn_append_pair(mpm_nn *net, cudaStream_t st, const double *r, const double *rr, const double *e);
int mpm_nn_grid_matches(const mpm_nn *net, const int nodes[3]);
