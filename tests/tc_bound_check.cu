// tc_bound_check.cu -- host-only soundness check of tc_error_bound, the
// certificate of the tensor form (csrc/tc.cuh).  Test infrastructure: built
// and run by tests/test_tc_bound.py on the CPU; nothing here touches a GPU.
//
// For seeded lists and queries in both operand formats the program restates,
// on the host, every quantity the engine derives for a (query, row) pair --
// the centered operands and their half-precision rounding, w (and its three
// BF16 pieces in the exact format), the query norm, the list bounds X and C,
// Dqr -- with the same roundings as the build and query kernels, and forms
// the tensor-core value under several models of the FP32 accumulation:
//   rz_step   each 16-term MMA step summed exactly, added with truncation
//   rz_each   every product added with truncation
//   rn_step   each step added with round-to-nearest
//   faithful  every product added with a random one of the two neighbours
// The exact distance is the reference's sequential FP32 sum of (q_i - x_i)^2
// (utils.cu:183-191, no FMA).  A pair violates the certificate when
// |approx - exact| > E; the program prints the pair count, the largest
// |approx - exact| / E per model and the violations, and exits 1 on any.
// Arguments: seed (default 1) and a factor applied to E (default 1; a small
// factor plants an underestimating bound, which the check must catch).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "tc.cuh"

using rbc::kTcExact;
using rbc::kTcSplit;

namespace {

constexpr int kModels = 4;
const char *kModelName[kModels] = {"rz_step", "rz_each", "rn_step", "faithful"};

float bf16_rn(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }
float fp16_rn(float v) { return __half2float(__float2half_rn(v)); }

// float nearest to x in the direction toward zero / away from zero
float to_zero(double x) {
  float f = (float)x;
  if (std::fabs((double)f) > std::fabs(x)) f = std::nextafter(f, 0.f);
  return f;
}
float away_zero(double x) {
  float f = (float)x;
  if (std::fabs((double)f) < std::fabs(x)) f = std::nextafter(f, x > 0 ? FLT_MAX : -FLT_MAX);
  return f;
}
float round_up(double x) {
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, FLT_MAX);
  return f;
}

// the reference's distance: sequential, multiply and add rounded separately
float seq_dist(const float *a, const float *b, int d) {
  float s = 0.f;
  for (int i = 0; i < d; i++) {
    const float t = a[i] - b[i];
    const float t2 = t * t;
    s = s + t2;
  }
  return s;
}

// a warp's strided FMA sums followed by the xor-shuffle tree (lanes 0..31)
float warp_fma_sum(const std::vector<float> &a, const std::vector<float> &b) {
  float lane[32];
  for (int l = 0; l < 32; l++) {
    float s = 0.f;
    for (size_t i = l; i < a.size(); i += 32) s = std::fma(a[i], b[i], s);
    lane[l] = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    float nxt[32];
    for (int l = 0; l < 32; l++) nxt[l] = lane[l] + lane[l ^ o];
    std::memcpy(lane, nxt, sizeof lane);
  }
  return lane[0];
}

float half_scale(float maxabs) {
  if (!(maxabs > 0.f)) return 1.f;
  int e = 13 - std::ilogb(maxabs);
  e = e < -120 ? -120 : (e > 120 ? 120 : e);
  return std::ldexp(1.f, e);
}

// One accumulator over a product list, in K-steps of 16 (products are exact
// in double: half x half values have at most 22 significant bits).
struct Acc {
  float v[kModels] = {0.f, 0.f, 0.f, 0.f};
  void step(const double *p, std::mt19937_64 &rng) {
    double s = 0.0;
    for (int t = 0; t < 16; t++) s += p[t];
    v[0] = to_zero((double)v[0] + s);
    v[2] = (float)((double)v[2] + s);
    for (int t = 0; t < 16; t++) {
      v[1] = to_zero((double)v[1] + p[t]);
      const double x = (double)v[3] + p[t];
      v[3] = (rng() & 1) ? to_zero(x) : away_zero(x);
    }
  }
};

struct Case {
  const char *name;
  uint32_t format;
  int d;
  int kind;  // data generator
};

struct Stats {
  long pairs = 0, viol = 0;
  double worst[kModels] = {0, 0, 0, 0};
};

// Rows of list r are c_r plus a perturbation; queries are near some list.
//   kind 0: geometric integer features (mean 20, clipped to 255), integer queries
//   kind 1: as 0 with fractional queries (inexact in BF16)
//   kind 2: integers times 2^e_i, e_i in [0, 12] per coordinate (wide range)
//   kind 3: integers around 2^20 (far from the origin: w is a large cancelling sum)
//   kind 4: Gaussian mixture in [0, 1]^d (split format)
//   kind 5: Gaussian values times 2^e_i, e_i in [-20, 20] (split format)
//   kind 6: Gaussian mixture around 1000 (split format, centering matters)
void make_data(const Case &cs, int nl, int per, int m, std::mt19937_64 &rng, std::vector<float> &C,
               std::vector<float> &X, std::vector<float> &Q) {
  const int d = cs.d;
  std::geometric_distribution<int> geo(1.0 / 21.0);
  std::normal_distribution<double> nrm(0.0, 1.0);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::vector<int> ex(d);
  for (int i = 0; i < d; i++) ex[i] = cs.kind == 2 ? (int)(rng() % 13) : (cs.kind == 5 ? (int)(rng() % 41) - 20 : 0);
  auto integer = [&](int i) {
    const double base = cs.kind == 3 ? 1048576.0 : 0.0;
    return (float)((base + std::min(geo(rng), 255)) * std::ldexp(1.0, ex[i]));
  };
  auto real = [&](int i, double centre) {
    const double sc = cs.kind == 5 ? std::ldexp(1.0, ex[i]) : 1.0;
    return (float)((centre + 0.05 * nrm(rng)) * sc);
  };
  C.assign((size_t)nl * d, 0.f);
  X.assign((size_t)nl * per * d, 0.f);
  Q.assign((size_t)m * d, 0.f);
  std::vector<double> centre((size_t)nl * d);
  for (auto &v : centre) v = (cs.kind == 6 ? 1000.0 : 0.0) + uni(rng);
  for (int r = 0; r < nl; r++)
    for (int i = 0; i < d; i++) C[(size_t)r * d + i] = cs.kind <= 3 ? integer(i) : real(i, centre[(size_t)r * d + i]);
  for (int r = 0; r < nl; r++)
    for (int p = 0; p < per; p++)
      for (int i = 0; i < d; i++) {
        float v;
        if (cs.kind <= 3) {
          // x = c + an integer step (scaled like the coordinate): x - c exact in BF16
          const int step = (int)(rng() % 255) - 127;
          v = C[(size_t)r * d + i] + (float)(step * std::ldexp(1.0, ex[i]));
          if (v < 0.f && cs.kind != 3) v = C[(size_t)r * d + i] - (float)(step * std::ldexp(1.0, ex[i]));
        } else {
          v = real(i, centre[(size_t)r * d + i]);
        }
        X[((size_t)r * per + p) * d + i] = v;
      }
  for (int q = 0; q < m; q++) {
    const int r = (int)(rng() % nl);
    for (int i = 0; i < d; i++) {
      float v;
      if (cs.kind <= 3) {
        v = integer(i);
        if (cs.kind == 1) v += (float)uni(rng);
        if (q % 4 == 0) v = C[(size_t)r * d + i] + (float)(((int)(rng() % 64) - 32) * std::ldexp(1.0, ex[i]));
      } else {
        v = real(i, centre[(size_t)r * d + i]);
      }
      Q[(size_t)q * d + i] = v;
    }
  }
}

void run_case(const Case &cs, uint64_t seed, float bound_factor, Stats &st) {
  const int d = cs.d, kp = (int)((d + 63) / 64 * 64), nl = 6, per = 48, m = 48;
  const bool split = cs.format == kTcSplit;
  std::mt19937_64 rng(seed);
  std::vector<float> C, X, Q;
  make_data(cs, nl, per, m, rng, C, X, Q);
  // mu: mean of the representatives (split format), zero in the exact format
  std::vector<float> mu(d, 0.f);
  if (split)
    for (int i = 0; i < d; i++) {
      double s = 0.0;
      for (int r = 0; r < nl; r++) s += C[(size_t)r * d + i];
      mu[i] = (float)(s / nl);
    }
  const double u = 5.9604644775390625e-08, g = (d + 3) * u / (1.0 - (d + 3) * u);
  // per list: x' operands, w, the bounds X (from the radius) and C
  std::vector<std::vector<float>> xop(nl * per), xop2(nl * per);
  std::vector<float> w(nl * per), Xb(nl), Cb(nl), ls(nl);
  uint32_t x_inexact = 0;
  for (int r = 0; r < nl; r++) {
    const float *c = &C[(size_t)r * d];
    float radius = 0.f, lmax = 0.f;
    for (int p = 0; p < per; p++) {
      const float *x = &X[((size_t)r * per + p) * d];
      radius = std::max(radius, seq_dist(x, c, d));
      for (int i = 0; i < d; i++) {
        const float v = x[i] - c[i];
        lmax = std::max(lmax, std::fabs(v));
        x_inexact |= bf16_rn(v) != v;
      }
    }
    ls[r] = split ? half_scale(lmax) : 1.f;
    Xb[r] = round_up(std::sqrt((double)radius / (1.0 - g)) * (1.0 + g));
    double cc = 0.0;
    for (int i = 0; i < d; i++) cc += ((double)c[i] - mu[i]) * ((double)c[i] - mu[i]);
    Cb[r] = round_up(std::sqrt(cc) * (1.0 + 4.0 * u));
  }
  if (!split && x_inexact) {
    std::fprintf(stderr, "%s: data not exact in BF16\n", cs.name);
    std::exit(2);
  }
  for (int r = 0; r < nl; r++)
    for (int p = 0; p < per; p++) {
      const float *x = &X[((size_t)r * per + p) * d], *c = &C[(size_t)r * d];
      std::vector<float> v(kp, 0.f), cm(kp, 0.f), hi(kp, 0.f), lo(kp, 0.f);
      for (int i = 0; i < d; i++) {
        v[i] = x[i] - c[i];
        cm[i] = c[i] - mu[i];
        if (split) {
          const float sv = v[i] * ls[r];
          hi[i] = fp16_rn(sv);
          lo[i] = fp16_rn(sv - hi[i]);
        } else {
          hi[i] = bf16_rn(v[i]);
        }
      }
      w[r * per + p] = warp_fma_sum(v, v) + 2.f * warp_fma_sum(cm, v);
      xop[r * per + p] = hi;
      xop2[r * per + p] = lo;
    }
  for (int q = 0; q < m; q++) {
    const float *qv = &Q[(size_t)q * d];
    std::vector<float> v(kp, 0.f), hi(kp, 0.f), lo(kp, 0.f);
    float mx = 0.f;
    uint32_t bad = 0;
    for (int i = 0; i < d; i++) {
      v[i] = qv[i] - mu[i];
      mx = std::max(mx, std::fabs(v[i]));
      bad |= bf16_rn(v[i]) != v[i];
    }
    const float t = split ? half_scale(mx) : 1.f;
    for (int i = 0; i < d; i++) {
      if (split) {
        const float sv = v[i] * t;
        hi[i] = fp16_rn(sv);
        lo[i] = fp16_rn(sv - hi[i]);
      } else {
        hi[i] = bf16_rn(v[i]);
      }
    }
    const float qn = std::sqrt(warp_fma_sum(v, v)) * (1.f + 1e-6f);
    const uint32_t qinex = split ? 0u : bad;
    for (int r = 0; r < nl; r++) {
      const float dq = seq_dist(qv, &C[(size_t)r * d], d);
      const float E =
          bound_factor * rbc::tc_error_bound(dq, qn, Xb[r], Cb[r], qinex, x_inexact, cs.format, (uint32_t)d);
      for (int p = 0; p < per; p++) {
        const int row = r * per + p;
        const float exact = seq_dist(qv, &X[(size_t)row * d], d);
        const std::vector<float> &xh = xop[row], &xl = xop2[row];
        Acc a1, a2;
        double prod[16];
        for (int k0 = 0; k0 < kp; k0 += 16) {
          for (int t16 = 0; t16 < 16; t16++) prod[t16] = (double)hi[k0 + t16] * xh[k0 + t16];
          a1.step(prod, rng);
          if (split) {
            for (int t16 = 0; t16 < 16; t16++) prod[t16] = (double)hi[k0 + t16] * xl[k0 + t16];
            a2.step(prod, rng);
            for (int t16 = 0; t16 < 16; t16++) prod[t16] = (double)lo[k0 + t16] * xh[k0 + t16];
            a2.step(prod, rng);
          }
        }
        float approx[kModels];
        if (split) {
          const float alpha = -2.f / (t * ls[r]);
          for (int md = 0; md < kModels; md++) {
            float tv = std::fma(alpha, a1.v[md], w[row]);
            tv = std::fma(alpha, a2.v[md], tv);
            approx[md] = dq + tv;
          }
        } else {
          // the folded w step: pieces w1 w2 w3 (twice) against -1/4
          const float wv = w[row];
          const float b1 = bf16_rn(wv), r1 = wv - b1, b2 = bf16_rn(r1), b3 = bf16_rn(r1 - b2);
          const double pc[3] = {-0.25 * b1, -0.25 * b2, -0.25 * b3};
          for (int t16 = 0; t16 < 16; t16++) prod[t16] = (t16 & 7) < 3 ? pc[t16 & 7] : 0.0;
          a1.step(prod, rng);
          for (int md = 0; md < kModels; md++) approx[md] = dq + -2.f * a1.v[md];
        }
        st.pairs++;
        for (int md = 0; md < kModels; md++) {
          const double err = std::fabs((double)approx[md] - (double)exact);
          if (!(err <= E)) {
            if (st.viol < 10)
              std::printf("violation %s model %s q %d row %d: approx %.9g exact %.9g err %.3g E %.3g\n", cs.name,
                          kModelName[md], q, row, approx[md], exact, err, E);
            st.viol++;
          }
          st.worst[md] = std::max(st.worst[md], err / E);
        }
      }
    }
  }
}

}  // namespace

int main(int argc, char **argv) {
  const uint64_t seed = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;
  const float bound_factor = argc > 2 ? std::strtof(argv[2], nullptr) : 1.f;
  const Case cases[] = {
      {"bf16_geometric_d128", kTcExact, 128, 0},   {"bf16_fractional_queries_d128", kTcExact, 128, 1},
      {"bf16_wide_range_d64", kTcExact, 64, 2},    {"bf16_far_from_origin_d128", kTcExact, 128, 3},
      {"bf16_geometric_d40", kTcExact, 40, 0},     {"split_mixture_d128", kTcSplit, 128, 4},
      {"split_wide_range_d32", kTcSplit, 32, 5},   {"split_far_from_origin_d96", kTcSplit, 96, 6},
  };
  long viol = 0;
  for (const Case &cs : cases) {
    Stats st;
    for (uint64_t s = 0; s < 3; s++) run_case(cs, seed * 1000 + s, bound_factor, st);
    std::printf("%s pairs %ld violations %ld worst", cs.name, st.pairs, st.viol);
    for (int md = 0; md < kModels; md++) std::printf(" %s=%.4g", kModelName[md], st.worst[md]);
    std::printf("\n");
    viol += st.viol;
  }
  std::printf("total violations %ld\n", viol);
  return viol ? 1 : 0;
}
