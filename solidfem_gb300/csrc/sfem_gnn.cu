// Launchers of the learned-preconditioner kernels (sfem_gnn_kernels.cuh).
#include <algorithm>

#include "sfem_internal.h"
#include "sfem_gnn_kernels.cuh"

namespace sfem {
namespace gnn {

static int blocks_for(int64_t n, int per) {
  int64_t b = (n + per - 1) / per;
  return (int)(b < 1 ? 1 : b);
}

template <bool WGRAD, typename GT>
static void layer_bwd(const Graph& g, const __nv_bfloat16* hin, const GT* Gout, const __nv_bfloat16* Wt, float* Gself,
                      float* Gmsg, float* partial, const int* done, cudaStream_t st) {
  constexpr size_t smem = layer_bwd_smem(WGRAD);
  static bool attr = false;  // per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_gnn_layer_bwd<WGRAD, GT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  count_launch();
  k_gnn_layer_bwd<WGRAD, GT><<<blocks_for(g.n, TILE), LT, smem, st>>>(g, hin, Gout, Wt, Gself, Gmsg, partial, done);
}

void launch_encode(const Graph& g, const float* v, const float* dinv, const float* params, __nv_bfloat16* h0,
                   float* xout, const int* done, cudaStream_t st) {
  count_launch();
  k_gnn_encode<<<blocks_for(g.n * 32, 256), 256, 0, st>>>(g.n, v, dinv, params, h0, xout, done);
}

void launch_layers_fwd(const Graph& g, const __nv_bfloat16* Wb, __nv_bfloat16* const* h, const int* done,
                       cudaStream_t st) {
  for (int l = 0; l < NL; l++) {
    count_launch();
    k_gnn_layer_fwd<<<blocks_for(g.n, TILE), LT, 0, st>>>(g, h[l], Wb + (size_t)l * H * AIN, h[l + 1], done);
  }
}

static int inf_grid(int64_t n) {
  static int cap = 0;  // resident CTAs of the layer kernel on this device
  if (cap == 0) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gnn_layer_inf<false, false, false>, LT, 0);
    cap = std::max(1, sms) * std::max(1, per);
  }
  const int64_t tiles = (n + TILE - 1) / TILE;
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, cap));
}

void launch_apply(const Graph& g, const float* r, const float* dinv, const float* params, const __nv_bfloat16* Wb,
                  __nv_bfloat16* const* h, float* out, const int* done, cudaStream_t st) {
  const size_t per = (size_t)H * AIN;
  const __nv_bfloat16* Wsb = Wb + 2 * NL * per;
  const int grid = inf_grid(g.n);
  static_assert(NL == 3, "the launch sequence below is written for three layers");
  // S: h1 = L1(We x), h2, h3
  count_launch();
  k_gnn_layer_inf<true, false, false><<<grid, LT, 0, st>>>(g, nullptr, r, dinv, params, Wb, h[1], nullptr, done);
  count_launch();
  k_gnn_layer_inf<false, false, false><<<grid, LT, 0, st>>>(g, h[1], r, dinv, params, Wb + per, h[2], nullptr, done);
  count_launch();
  k_gnn_layer_inf<false, false, false><<<grid, LT, 0, st>>>(g, h[2], r, dinv, params, Wb + 2 * per, h[3], nullptr,
                                                              done);
  // S^T: L3^T h3 -> h[1], L2^T -> h[2], L1^T and We^T -> out
  count_launch();
  k_gnn_layer_inf<false, true, false><<<grid, LT, 0, st>>>(g, h[3], r, dinv, params, Wsb + 2 * per, h[1], nullptr,
                                                             done);
  count_launch();
  k_gnn_layer_inf<false, true, false><<<grid, LT, 0, st>>>(g, h[1], r, dinv, params, Wsb + per, h[2], nullptr, done);
  count_launch();
  k_gnn_layer_inf<false, true, true><<<grid, LT, 0, st>>>(g, h[2], r, dinv, params, Wsb, nullptr, out, done);
}

void launch_apply_poly(const Graph& g, const float* r, const float* dinv, const PolyCoef& pc, Row16* x4, Row16* y1,
                       Row16* y2, Row16* w, float* xstat, float* out, const int* done, cudaStream_t st,
                       float* partials, unsigned* counter, const float* rprev, CgScalars* s, bool x_ready,
                       CoarseAdd ca, cudaEvent_t before_last) {
  static_assert(NL == 3, "the launch sequence below is written for three layers");
  // grid-stride passes sized to one resident wave (no partly filled last wave; the BETA pass
  // then finishes with one block partial per resident CTA, 4 values each)
  static const int wave_fwd = resident_ctas(k_poly_fwd, 256, 0), wave_mid = resident_ctas(k_poly_mid, 256, 0),
                   wave_bwd = resident_ctas(k_poly_bwd, 256, 0),
                   wave_last = std::min(resident_ctas(k_poly_last<true>, 256, 0),
                                        resident_ctas(k_poly_last<false>, 256, 0));
  const int blocks = blocks_for(g.n, 256);
  if (!x_ready) launch_scale_sqrt4(g.n, r, dinv, xstat, partials, counter, x4, st);
  count_launch();
  launch_pdl(k_poly_fwd, std::min(blocks, wave_fwd), 256, 0, st, g, (const Row16*)x4, y1, done);
  count_launch();
  launch_pdl(k_poly_fwd, std::min(blocks, wave_fwd), 256, 0, st, g, (const Row16*)y1, y2, done);
  count_launch();
  launch_pdl(k_poly_mid, std::min(blocks, wave_mid), 256, 0, st, g, (const Row16*)x4, (const Row16*)y1,
             (const Row16*)y2, pc, w, done);
  // Horner in A^T: w3 -> A^T u + w2 (into y1) -> A^T u + w1 (into y2) -> out
  count_launch();
  launch_pdl(k_poly_bwd, std::min(blocks, wave_bwd), 256, 0, st, g, (const Row16*)(w + 3 * g.n),
             (const Row16*)(w + 2 * g.n), y1, done);
  count_launch();
  launch_pdl(k_poly_bwd, std::min(blocks, wave_bwd), 256, 0, st, g, (const Row16*)y1, (const Row16*)(w + g.n), y2,
             done);
  if (before_last) cudaStreamWaitEvent(st, before_last, 0);
  count_launch();
  const int grid_last = std::min(blocks, wave_last);
  if (s)
    launch_pdl(k_poly_last<true>, grid_last, 256, 0, st, g, (const Row16*)y2, (const Row16*)w, (const float*)xstat,
               r, dinv, pc.c, out, done, rprev, partials, counter, s, ca);
  else
    launch_pdl(k_poly_last<false>, grid_last, 256, 0, st, g, (const Row16*)y2, (const Row16*)w, (const float*)xstat,
               r, dinv, pc.c, out, done, nullptr, nullptr, nullptr, nullptr, ca);
}

// the training forward: activations h0..h3 of S at x (kept, with x), then S^T through the
// weight-gradient kernels' propagation; the same M(r) as launch_apply up to BF16 rounding
void launch_apply_train(const Graph& g, const float* r, const float* dinv, const float* params,
                        const __nv_bfloat16* Wb, __nv_bfloat16* const* h, float* x, float* G0, float* G1, float* G2,
                        float* out, cudaStream_t st) {
  const __nv_bfloat16* Wtb = Wb + (size_t)NL * H * AIN;
  launch_encode(g, r, dinv, params, h[0], x, nullptr, st);
  launch_layers_fwd(g, Wb, h, nullptr, st);
  const int nsc = blocks_for(g.n * 32, 256);
  layer_bwd<false, __nv_bfloat16>(g, nullptr, h[NL], Wtb + (size_t)(NL - 1) * H * AIN, G1, G2, nullptr, nullptr, st);
  count_launch();
  k_gnn_msg_scatter<<<nsc, 256, 0, st>>>(g, G1, G2, G0, nullptr);
  for (int l = NL - 2; l >= 0; l--) {
    layer_bwd<false, float>(g, nullptr, G0, Wtb + (size_t)l * H * AIN, G1, G2, nullptr, nullptr, st);
    count_launch();
    k_gnn_msg_scatter<<<nsc, 256, 0, st>>>(g, G1, G2, G0, nullptr);
  }
  count_launch();
  k_gnn_decode<<<nsc, 256, 0, st>>>(g.n, G0, params, r, dinv, out, nullptr);
}

int launch_count_apply() { return 2 * NL; }

void launch_weight_grad(const Graph& g, const __nv_bfloat16* cot, __nv_bfloat16* const* h, const float* x,
                        const __nv_bfloat16* Wb, float* G0, float* G1, float* G2, float* partial, float* grad,
                        int accumulate, cudaStream_t st) {
  const __nv_bfloat16* Wtb = Wb + (size_t)NL * H * AIN;
  const int nbl = blocks_for(g.n, TILE), nsc = blocks_for(g.n * 32, 256);
  for (int l = NL - 1; l >= 0; l--) {
    // layer l maps h[l] -> h[l+1]; the cotangent of h[l+1] is cot (l = NL-1) or G0
    if (l == NL - 1)
      layer_bwd<true, __nv_bfloat16>(g, h[l], cot, Wtb + (size_t)l * H * AIN, G1, G2, partial, nullptr, st);
    else
      layer_bwd<true, float>(g, h[l], G0, Wtb + (size_t)l * H * AIN, G1, G2, partial, nullptr, st);
    count_launch();
    k_gnn_reduce_cols<<<(LPART + 255) / 256, 256, 0, st>>>(nbl, LPART, partial, grad + OFF_L + l * L_STRIDE,
                                                             accumulate);
    count_launch();
    k_gnn_msg_scatter<<<nsc, 256, 0, st>>>(g, G1, G2, G0, nullptr);
  }
  const int nbe = blocks_for(g.n, 64);
  count_launch();
  k_gnn_encode_bwd<<<nbe, 256, 0, st>>>(g.n, G0, x, partial);
  count_launch();
  k_gnn_reduce_cols<<<(H * FIN + 255) / 256, 256, 0, st>>>(nbe, H * FIN, partial, grad + OFF_WE, accumulate);
}

void launch_cgrad(int64_t n3, const float* Go, const float* r, const float* dinv, const float* params, float* partials,
                  unsigned* counter, float* grad, int accumulate, cudaStream_t st) {
  int grid = blocks_for(n3, 256);
  if (grid > 1024) grid = 1024;
  count_launch();
  k_gnn_cgrad<<<grid, 256, 0, st>>>(n3, Go, r, dinv, params, partials, counter, grad, accumulate);
}

void launch_loss(int64_t n3, const float* d, const float* q, float inv_c, float* Go, float* partials,
                 unsigned* counter, float* loss, cudaStream_t st) {
  int grid = blocks_for(n3, 256);
  if (grid > 1024) grid = 1024;
  count_launch();
  k_gnn_loss<<<grid, 256, 0, st>>>(n3, d, q, inv_c, Go, partials, counter, loss);
}

void launch_adam(const float* grad, float* prm, float* m, float* v, float lr, int t, float clip_scale,
                 __nv_bfloat16* Wb, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
  count_launch();
  k_gnn_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(NPARAM, prm, grad, m, v, lr, b1, b2, 1e-8f, bc1, bc2, clip_scale);
  launch_pack(prm, Wb, st);
}

void launch_pack(const float* prm, __nv_bfloat16* Wb, cudaStream_t st) {
  count_launch();
  k_gnn_pack<<<(NL * H * AIN + 255) / 256, 256, 0, st>>>(prm, Wb);
}

}  // namespace gnn
}  // namespace sfem

// ---------------------------------------------------------------------------
// Flexible CG vector kernels (FP32) and small helpers
// ---------------------------------------------------------------------------
namespace sfem {
namespace gnn {

// xs = sigma r D^-1/2 (the input of the polynomial passes): sigma from sum d r^2, then the rows
void launch_scale_sqrt4(int64_t n, const float* r, const float* dinv, float* xstat, float* partials, unsigned* counter,
                        Row16* x4, cudaStream_t st) {
  static const int wave = resident_ctas(k_poly_xscale, 256, 0);
  const int g3 = (int)std::max<int64_t>(1, std::min<int64_t>((3 * n + 255) / 256, wave));
  count_launch();
  launch_pdl(k_poly_xscale, g3, 256, 0, st, 3 * n, r, dinv, xstat, partials, counter);
  int grid = (int)std::min<int64_t>((n + 255) / 256, 2048);
  count_launch();
  launch_pdl(k_scale_sqrt4, grid < 1 ? 1 : grid, 256, 0, st, n, r, dinv, (const float*)xstat, x4);
}

// d = a - b
__global__ void k_sub(int64_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = a[i] - b[i];
}
void launch_sub(int64_t n, const float* a, const float* b, float* d, cudaStream_t st) {
  int grid = (int)std::min<int64_t>((n + 255) / 256, 2048);
  count_launch();
  k_sub<<<grid < 1 ? 1 : grid, 256, 0, st>>>(n, a, b, d);
}

// rz = r.z, p = 0, beta = 0 (the first direction is z itself), after the CG initialisation
// has set r, x, bb
__global__ void __launch_bounds__(256) k_fcg_init(int64_t n, const float* __restrict__ r, const float* __restrict__ z,
                                                  float* __restrict__ p, float* __restrict__ partials,
                                                  unsigned* counter, CgScalars* s) {
  float acc[1] = {0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    p[i] = 0.f;
    acc[0] += r[i] * z[i];
  }
  double t[1];
  if (last_block_sums<1>(acc, partials, counter, t) && threadIdx.x == 0) {
    s->rz = t[0];
    s->beta = 0.0;
    s->jac = 0;
  }
}

// Polak-Ribiere: beta = z.(r - rprev) / rz_old, rz = z.r.  The same sums are formed for the
// Jacobi direction z_J = D^-1 r; when the learned direction is not a descent direction
// (z.r <= 0) this iteration falls back to Jacobi (s->beta / s->rz refer to the chosen z and
// s->jac = 1 makes the next fused direction update use D^-1 r).  Used with the layer-kernel
// inference; the polynomial inference forms these sums in its last pass.
__global__ void __launch_bounds__(256) k_fcg_beta(int64_t n, const float* __restrict__ r,
                                                  const float* __restrict__ rprev, const float* __restrict__ z,
                                                  const float* __restrict__ dinv, float* __restrict__ partials,
                                                  unsigned* counter, CgScalars* s) {
  if (s->done) return;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = r[i];
    const float dr = ri - rprev[i];
    const float zj = dinv[i] * ri;
    acc[0] += z[i] * dr;
    acc[1] += z[i] * ri;
    acc[2] += zj * dr;
    acc[3] += zj * ri;
  }
  double t[4];
  if (!last_block_sums<4>(acc, partials, counter, t) || threadIdx.x != 0) return;
  const bool learned_ok = t[1] > 0.0 && isfinite(t[1]) && isfinite(t[0]);
  if (learned_ok) {
    s->beta = t[0] / s->rz;
    s->rz = t[1];
    s->jac = 0;
  } else {
    s->beta = t[2] / s->rz;
    s->rz = t[3];
    s->jac = 1;
  }
}

static int vgrid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 1024) b = 1024;
  return (int)b;
}
void launch_fcg_init(int64_t n, const float* r, const float* z, float* p, float* partials, unsigned* counter,
                     CgScalars* s, cudaStream_t st) {
  count_launch();
  k_fcg_init<<<vgrid(n), 256, 0, st>>>(n, r, z, p, partials, counter, s);
}
void launch_fcg_beta(int64_t n, const float* r, const float* rprev, const float* z, const float* dinv,
                     float* partials, unsigned* counter, CgScalars* s, cudaStream_t st) {
  count_launch();
  k_fcg_beta<<<vgrid(n), 256, 0, st>>>(n, r, rprev, z, dinv, partials, counter, s);
}

}  // namespace gnn
}  // namespace sfem
