// router.cuh -- the learned list router (router.cu).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace rbc {

// MLP d -> H -> H -> L with GELU; parameters flat [W1 b1 W2 b2 W3 b3], FP32
// master copy w, gradients g, Adam moments m1 m2, BF16 weight copy wb.  With
// a distance head (T = 1) W3 and b3 carry one more output row: a regression
// of the normalised log ratio of the query's k-th neighbour distance to its
// nearest representative's, log (tau / near) = tau_mu + tau_sigma (z + tau_margin).
struct Router {
  uint32_t d = 0, H = 0, L = 0, T = 0;
  float tau_mu = 0.f, tau_sigma = 1.f, tau_margin = 0.f;
  const float *tau_src = nullptr;  // training: normalised targets of the whole set (NaN: none)
  float *yt = nullptr, *zt = nullptr;  // batch: targets, head outputs (their gradients after backward)
  float *w = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
  __nv_bfloat16 *wb = nullptr;
  uint64_t step = 0;
  // batch workspace
  uint32_t cap = 0;
  float *X = nullptr;
  uint32_t *y = nullptr;
  float *h1 = nullptr, *a1 = nullptr, *h2 = nullptr, *a2 = nullptr, *z = nullptr, *ga = nullptr, *gb = nullptr,
        *loss = nullptr;

  size_t nparams() const;
  cudaError_t init(uint64_t seed, cudaStream_t s);
  cudaError_t alloc_batch(uint32_t b, cudaStream_t s);
  cudaError_t gather(const float *Q, uint32_t ldq, const uint32_t *order, const uint32_t *labels, uint32_t b,
                     cudaStream_t s);
  // logits (z, b x L) and / or the distance head's outputs (zt_out, b), either may be null
  cudaError_t forward(const float *X, uint32_t ldx, uint32_t b, float *z, cudaStream_t s, float *zt_out = nullptr);
  cudaError_t forward_backward(uint32_t b, cudaStream_t s);
  cudaError_t adam_step(float lr, cudaStream_t s);
  cudaError_t refresh_bf16(cudaStream_t s);
  // inference on the tensor cores (router_tc.cu): needs H a multiple of 64
  uint64_t version = 0;  // bumped whenever the BF16 weights change
  uint32_t tc_cap = 0;
  __nv_bfloat16 *xb = nullptr, *h1b = nullptr, *h2b = nullptr, *w1p = nullptr;
  uint64_t w1p_version = ~0ull;
  bool tc_ok() const;
  // the probe table straight from the hidden activations (the last layer
  // fused with the top-P selection, no logits written): when top_ok(P + Pn)
  bool top_ok(uint32_t width) const;
  cudaError_t probes_tc(const float *X, uint32_t ldx, uint32_t b, uint32_t P, uint32_t Pn, const uint32_t *nearest,
                        const float *nearest_d, uint32_t *probe, float *probed, uint32_t *err, cudaStream_t s);
  cudaError_t forward_tc(const float *X, uint32_t ldx, uint32_t b, float *z, uint32_t *err, cudaStream_t s);
  // the distance head alone: its outputs, and the predicted k-th distances
  // (distance units, margin included)
  cudaError_t head_outputs(const float *X, uint64_t ldx, uint64_t b, float *zt_out, uint32_t *err, cudaStream_t s);
  cudaError_t predict_tau(const float *X, uint32_t ldx, uint32_t b, const float *near, float *tau, uint32_t *err,
                          cudaStream_t s);
  cudaError_t forward_tc_head(const float *X, uint32_t ldx, uint32_t b, float *zt_out, uint32_t *err,
                              cudaStream_t s);
  ~Router();
};

// Probe table of width Pn + P: the Pn nearest representatives (a Pn-wide
// table, nearest first) then the top-P lists of each row of router logits not
// among them (largest first, ties to the lower list).  Pn + P <= 16.
cudaError_t launch_router_probes(const float *logits, uint64_t m, uint32_t L, uint32_t P, uint32_t Pn,
                                 const uint32_t *nearest, const float *nearest_d, uint32_t *probe, float *probed,
                                 cudaStream_t s);
// tau[i] = near[i] exp(mu + sigma (z[i] + margin)), nudged up (a prediction, not a bound)
cudaError_t launch_tau_from_head(const float *z, const float *near, uint64_t m, float mu, float sigma, float margin,
                                 float *tau, cudaStream_t s);
// labels[i] = owner[ids[i]]
cudaError_t launch_owner_lookup(const uint32_t *ids, uint64_t m, uint32_t ldo, const uint32_t *owner,
                                uint32_t *labels, cudaStream_t s);

}  // namespace rbc

struct rbc_router {
  rbc::Router r;
};
