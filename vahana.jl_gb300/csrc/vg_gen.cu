// Seeded graph generators of the test models (device side) and read-back of
// staged edge records.  A generator plays the part of the model script's
// add_edge! loop before finish_init!: it appends records in the loop's call
// order to the edge type's staging, exactly as that many add_edge! calls
// would (src/EdgeMethods.jl:478-522); finish_init! then builds the CSR.
#include <algorithm>
#include <cmath>
#include <vector>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n) { return (unsigned)std::max<uint64_t>((n + TPB - 1) / TPB, 1); }

// uniform out-edges: agent i (1-based) adds k edges i -> t, t uniform in
// [1, N] without self loops (t >= i -> t + 1), in the order (i, j).
__global__ void k_gen_uniform_out(uint64_t N, uint32_t k, uint64_t seed, int type_nr,
                                  uint64_t first_nr, uint64_t *from, uint64_t *to) {
  uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N * k) return;
  uint64_t i = r / k + 1;
  uint32_t j = (uint32_t)(r % k) + 1;
  Philox4 p = philox_draw(seed, i, j, TAG_EDGE);
  uint64_t t = (uint64_t)bounded32(p.v[0], (uint32_t)(N - 1)) + 1;
  if (t >= i) t += 1;
  from[r] = ((uint64_t)type_nr << SHIFT_TYPE) | (first_nr + i - 1);
  to[r] = ((uint64_t)type_nr << SHIFT_TYPE) | (first_nr + t - 1);
}

// smallest index i with cdf[i] > u (cdf inclusive prefix sums of weights)
// first i in [lo, hi] with cdf[i] > u, else hi.  The cdf and u are
// non-negative finite doubles, whose order is the order of their bit
// patterns as unsigned integers: the comparisons run on the integer pipes
// (the binary64 pipe of this GPU is 64x narrower) with the same outcome.
__device__ __forceinline__ uint64_t sample_cdf_in(const double *cdf, uint64_t lo, uint64_t hi,
                                                  double u) {
  const unsigned long long ub = (unsigned long long)__double_as_longlong(u);
  const long long *cb = reinterpret_cast<const long long *>(cdf);
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if ((unsigned long long)cb[mid] > ub) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ uint64_t sample_cdf(const double *cdf, uint64_t n, double u) {
  return sample_cdf_in(cdf, 0, n - 1, u);
}

// guide table: guide[b] = sample_cdf(b * total / G), b = 0..G.  The sample
// of u lies between the entries of the buckets around u * G / total
// (widened by one bucket on each side against rounding of the bucket
// index), so the search over that range returns the full search's index.
constexpr uint32_t GUIDE_BITS = 20;
__global__ void k_cdf_guide(const double *cdf, uint64_t n, double total, uint32_t *guide) {
  uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t G = 1ull << GUIDE_BITS;
  if (b > G) return;
  guide[b] = (uint32_t)sample_cdf(cdf, n, (double)b * (total / (double)G));
}

__device__ __forceinline__ uint64_t sample_guided(const double *cdf, const uint32_t *guide,
                                                  double total, double u) {
  const uint64_t G = 1ull << GUIDE_BITS;
  double fb = u * ((double)G / total);
  uint64_t b = fb <= 0.0 ? 0 : (fb >= (double)G ? G - 1 : (uint64_t)fb);
  const uint64_t lo = guide[b > 0 ? b - 1 : 0];
  const uint64_t hi = guide[b + 2 <= G ? b + 2 : G];
  return sample_cdf_in(cdf, lo, hi, u);
}

// directed Chung-Lu: edge e draws source and target proportional to the
// expected degrees and a weight in (0, 1]
__global__ void k_gen_chung_lu(uint64_t E, const double *cdf, const uint32_t *guide,
                               double total, uint64_t seed, int type_nr, uint64_t first_nr,
                               uint64_t *from, uint64_t *to, double *w) {
  uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  double us = u64_to_unit(philox_u64(philox_draw(seed, e, 0, TAG_SRC))) * total;
  double ud = u64_to_unit(philox_u64(philox_draw(seed, e, 0, TAG_DST))) * total;
  uint64_t s = sample_guided(cdf, guide, total, us), d = sample_guided(cdf, guide, total, ud);
  from[e] = ((uint64_t)type_nr << SHIFT_TYPE) | (first_nr + s);
  to[e] = ((uint64_t)type_nr << SHIFT_TYPE) | (first_nr + d);
  if (w) w[e] = u64_to_unit_open0(philox_u64(philox_draw(seed, e, 0, TAG_WEIGHT)));
}

EdgeSegment &new_device_segment(Sim &s, int e, uint64_t n) {
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  if (es.implicit) fail(VG_ERR_ARG, "edge type holds implicit raster edges");
  EdgeSegment seg;
  seg.device = true;
  seg.n = n;
  seg.d_from.alloc(std::max<uint64_t>(n, 1) * 8, &s.footprint);
  seg.d_to.alloc(std::max<uint64_t>(n, 1) * 8, &s.footprint);
  int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
  seg.d_payload.resize(nf);
  for (int f = 0; f < nf; f++) {
    seg.d_payload[f].alloc(std::max<uint64_t>(n, 1) * ed.fields[f].size, &s.footprint);
    VG_CUDA(cudaMemsetAsync(seg.d_payload[f].p, 0, std::max<uint64_t>(n, 1) * ed.fields[f].size, s.stream));
  }
  es.staged.push_back(std::move(seg));
  es.nstaged += n;
  return es.staged.back();
}

}  // namespace

// expected degrees w_i = min(c * i^(-1/(gamma-1)), wmax) with c chosen so that
// the mean is `mean` (bisection on the capped sum)
std::vector<double> chung_lu_weights(uint64_t N, double mean, double gamma, double wmax) {
  std::vector<double> r(N), suffix(N + 1, 0.0);
  double ex = -1.0 / (gamma - 1.0);
  for (uint64_t i = 0; i < N; i++) r[i] = std::pow((double)(i + 1), ex);
  for (uint64_t i = N; i-- > 0;) suffix[i] = suffix[i + 1] + r[i];
  auto capped_sum = [&](double c) {
    // r is decreasing: the first k entries are capped
    uint64_t lo = 0, hi = N;  // k = number of i with c * r[i] >= wmax
    while (lo < hi) {
      uint64_t mid = (lo + hi) / 2;
      if (c * r[mid] >= wmax) lo = mid + 1; else hi = mid;
    }
    return wmax * (double)lo + c * suffix[lo];
  };
  double target = mean * (double)N, lo = 0.0, hi = wmax / r[N - 1];
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    if (capped_sum(mid) < target) lo = mid; else hi = mid;
  }
  double c = 0.5 * (lo + hi);
  std::vector<double> w(N);
  for (uint64_t i = 0; i < N; i++) w[i] = std::min(c * r[i], wmax);
  return w;
}

}  // namespace vg

using namespace vg;

namespace vg {
void set_last_error(const std::string &m);
}

#define API_BEGIN try {
#define API_END                     \
  return VG_OK;                     \
  }                                 \
  catch (const Error &e) {          \
    set_last_error(e.msg);          \
    return e.code;                  \
  }                                 \
  catch (const std::exception &e) { \
    set_last_error(e.what());       \
    return VG_ERR_ARG;              \
  }

static Sim &S(vg_sim *s) {
  if (!s || !s->s) fail(VG_ERR_ARG, "null simulation handle");
  return *s->s;
}

extern "C" {

int vg_gen_uniform_out_edges(vg_sim *h, int e, int type_nr, uint32_t k, uint64_t seed) {
  API_BEGIN
  Sim &s = S(h);
  if (s.initialized) fail(VG_ERR_ASSERT, "generators run before finish_init!");
  s.ensure_device();
  AgentStore &a = s.agents[type_nr - 1];
  uint64_t N = a.h_n;
  if (N < 2) fail(VG_ERR_ARG, "need at least two agents");
  if (N > 0xffffffffull) fail(VG_ERR_ARG, "uniform generator: at most 2^32 agents");
  EdgeSegment &seg = new_device_segment(s, e, N * k);
  k_gen_uniform_out<<<nblk(N * k), TPB, 0, s.stream>>>(N, k, seed, type_nr, 1,
                                                       seg.d_from.as<uint64_t>(),
                                                       seg.d_to.as<uint64_t>());
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

int vg_gen_chung_lu_edges(vg_sim *h, int e, int type_nr, uint64_t nedges, double mean,
                          double gamma, double wmax, uint64_t seed, int weight_field) {
  API_BEGIN
  Sim &s = S(h);
  if (s.initialized) fail(VG_ERR_ASSERT, "generators run before finish_init!");
  s.ensure_device();
  const EdgeTypeDesc &ed = s.model->et(e);
  AgentStore &a = s.agents[type_nr - 1];
  uint64_t N = a.h_n;
  if (N < 1) fail(VG_ERR_ARG, "no agents");
  std::vector<double> w = chung_lu_weights(N, mean, gamma, wmax);
  std::vector<double> cdf(N);
  double acc = 0;
  for (uint64_t i = 0; i < N; i++) {
    acc += w[i];
    cdf[i] = acc;
  }
  double *d_cdf = nullptr;
  VG_CUDA(cudaMallocAsync((void **)&d_cdf, N * 8, s.stream));
  VG_CUDA(cudaMemcpyAsync(d_cdf, cdf.data(), N * 8, cudaMemcpyHostToDevice, s.stream));
  EdgeSegment &seg = new_device_segment(s, e, nedges);
  double *wp = nullptr;
  if (weight_field >= 0) {
    if (!ed.stores_payload() || weight_field >= (int)ed.fields.size() ||
        ed.fields[weight_field].dtype != VG_F64)
      fail(VG_ERR_ARG, "weight field must be a Float64 edge field");
    wp = seg.d_payload[weight_field].as<double>();
  }
  uint32_t *d_guide = nullptr;
  const uint64_t G = 1ull << GUIDE_BITS;
  VG_CUDA(cudaMallocAsync((void **)&d_guide, (G + 1) * 4, s.stream));
  k_cdf_guide<<<nblk(G + 1), TPB, 0, s.stream>>>(d_cdf, N, acc, d_guide);
  k_gen_chung_lu<<<nblk(nedges), TPB, 0, s.stream>>>(nedges, d_cdf, d_guide, acc, seed, type_nr, 1,
                                                     seg.d_from.as<uint64_t>(),
                                                     seg.d_to.as<uint64_t>(), wp);
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaFreeAsync(d_guide, s.stream));
  VG_CUDA(cudaFreeAsync(d_cdf, s.stream));
  VG_CUDA(cudaStreamSynchronize(s.stream));
  API_END
}

// Staged (not yet built) edge records of one edge type, in call order.
int vg_read_staged_edges(vg_sim *h, int e, uint64_t *from_out, uint64_t *to_out,
                         void *const *payload_out, uint64_t cap, uint64_t *n_out) {
  API_BEGIN
  need(n_out, "count pointer");
  Sim &s = S(h);
  const EdgeTypeDesc &ed = s.model->et(e);
  EdgeStore &es = s.edges[e];
  uint64_t n = 0;
  for (auto &sg : es.staged) n += sg.n;
  *n_out = n;
  uint64_t off = 0;
  int nf = ed.stores_payload() ? (int)ed.fields.size() : 0;
  for (auto &sg : es.staged) {
    uint64_t m = std::min<uint64_t>(sg.n, cap > off ? cap - off : 0);
    if (!m) break;
    if (sg.device) {
      if (from_out) VG_CUDA(cudaMemcpyAsync(from_out + off, sg.d_from.p, m * 8, cudaMemcpyDeviceToHost, s.stream));
      if (to_out) VG_CUDA(cudaMemcpyAsync(to_out + off, sg.d_to.p, m * 8, cudaMemcpyDeviceToHost, s.stream));
      for (int f = 0; f < nf; f++)
        if (payload_out && payload_out[f])
          VG_CUDA(cudaMemcpyAsync((uint8_t *)payload_out[f] + off * ed.fields[f].size,
                                  sg.d_payload[f].p, m * ed.fields[f].size,
                                  cudaMemcpyDeviceToHost, s.stream));
      VG_CUDA(cudaStreamSynchronize(s.stream));
    } else {
      if (from_out) std::copy(sg.h_from.begin(), sg.h_from.begin() + m, from_out + off);
      if (to_out) std::copy(sg.h_to.begin(), sg.h_to.begin() + m, to_out + off);
      for (int f = 0; f < nf; f++)
        if (payload_out && payload_out[f])
          std::copy(sg.h_payload[f].begin(), sg.h_payload[f].begin() + m * ed.fields[f].size,
                    (uint8_t *)payload_out[f] + off * ed.fields[f].size);
    }
    off += m;
  }
  API_END
}

}  // extern "C"
