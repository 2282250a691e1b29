// Sizes, parameter layout and plain structs of the learned preconditioner, shared by
// the host driver and the kernels (sfem_gnn_kernels.cuh).
#pragma once
#include <stdint.h>

namespace sfem {
namespace gnn {

constexpr int H = 64;        // width
constexpr int FIN = 3;       // input channels: D^-1/2 r at one node
constexpr int NL = 3;        // message-passing layers
constexpr int AIN = 2 * H;   // layer input [h ; mean h]
constexpr int TILE = 64;     // nodes per CTA in the layer kernels
constexpr int LT = 128;      // threads per CTA in the layer kernels (4 warps x 16 nodes)
constexpr int SROW = AIN + 8;  // padded shared-memory row (bf16) for 128-wide rows
constexpr int SROW64 = H + 8;  // padded row for 64-wide rows

// parameter vector layout (FP32 master copy)
constexpr int OFF_WE = 0;                      // We [H x FIN]
constexpr int OFF_L = OFF_WE + H * FIN;        // per layer: Wl [H x AIN]
constexpr int L_STRIDE = H * AIN;
constexpr int OFF_C = OFF_L + NL * L_STRIDE;   // log c (weight of the Jacobi term)
constexpr int NPARAM = OFF_C + 1;
constexpr int LPART = H * AIN;  // per-CTA partial of one layer's weight gradient

// The network folded into its polynomial form (S is linear and its feature maps commute with
// the node aggregation A):  S^T S x = sum_{j,k} (A^T)^j (A^k x) G[k][j],  G[k][j] 3 x 3.
struct PolyCoef {
  float G[NL + 1][NL + 1][9];  // row-major: w_j += y_k G[k][j] (row vector y_k)
  float c;                     // weight of the Jacobi term
};

// A node row of the polynomial passes: (x, y, z) in FP16 and a zero pad, 8 bytes.  The rows hold
// the polynomial's input D^-1/2 r (and what the passes make of it) times a power of two, sigma, that
// puts their RMS in [1/8, 1/4): xstat[0] is the sum of d r^2 over the last rows formed, xstat[1]
// their sigma, which the last pass divides out.
struct alignas(8) Row16 {
  uint32_t xy, z0;
};

struct Graph {
  int64_t n;              // free nodes
  const int32_t* ptr;     // n + 1
  const int32_t* idx;     // neighbours (free-node indices)
  const float* inv_deg;   // 1 / max(deg, 1)
  const int16_t* d16;     // the same neighbours as j - i when every |j - i| < 2^15 (else null)
  // neighbour patterns (else null): node i's deltas j - i are ptab[pptr[pid[i]] .. pptr[pid[i] + 1])
  const uint16_t* pid;
  const int32_t* pptr;
  const int16_t* ptab;
};


}  // namespace gnn
}  // namespace sfem
