// vg_sir_step_noalloc: one SIR transition step on buffers the caller owns,
// for callers that cannot allocate device memory (a host runtime that hands
// the library pre-allocated device arrays and forbids allocation, or code
// that runs while another framework captures a CUDA graph and must not
// allocate).  The entry point allocates nothing: its only scratch -- the
// table of infection probabilities p_k = 1 - (1 - beta)^k -- lives in a
// file-scope device array of fixed size.
//
// Shared scratch: every call writes the same array.  Calls whose work
// overlaps on the GPU (different streams, or different host threads) race
// on it and must be serialised by the caller.  Each call rewrites entries
// 0..max_in_degree before its step kernel reads them (stream order), so
// nothing has to start at zero.
//
// Set-up: the first call on a device, with that device current, looks up
// the array's device address (cudaGetSymbolAddress) once and caches it per
// device; make that first call before any stream capture.
#include <mutex>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
namespace {

constexpr int NOALLOC_MAX_DEGREE = 4095;  // largest in-degree the table covers
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_sir_ptab[NOALLOC_MAX_DEGREE + 1];

double *g_ptab_addr[MAX_DEVICES] = {nullptr};
std::mutex g_setup_mutex;

// p_k = 1 - q_k with q_k = q_{k-1} * (1 - beta), k = 0..kmax, computed by
// one thread in this order (the same sequence of roundings as the host table
// of the "sir" transition)
__global__ void k_fill_ptab(double *tab, uint32_t kmax, double beta) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double q = 1.0, om = 1.0 - beta;
  tab[0] = 0.0;
  for (uint32_t k = 1; k <= kmax; k++) {
    q = q * om;
    tab[k] = 1.0 - q;
  }
}

__global__ void k_sir_noalloc(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ src,
                              const uint8_t *__restrict__ st_rd, const int32_t *__restrict__ d_rd,
                              uint8_t *__restrict__ st_wr, int32_t *__restrict__ d_wr, uint64_t n,
                              const double *__restrict__ tab, uint32_t kmax, double beta,
                              uint64_t seed, uint32_t step, int32_t recovery) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t s = st_rd[i];
  int32_t d = d_rd[i];
  if (s == 0) {
    uint32_t k = 0;
    uint32_t e = rp[i + 1];
    for (uint32_t q = rp[i]; q < e; q++) k += (__ldg(st_rd + src[q]) == 1);
    if (k > 0) {
      double p;
      if (k <= kmax) {
        p = tab[k];
      } else {  // beyond the table: the same product, computed here
        double q = 1.0, om = 1.0 - beta;
        for (uint32_t j = 0; j < k; j++) q = q * om;
        p = 1.0 - q;
      }
      double u = u64_to_unit(philox_u64(philox_draw(seed, i + 1, step, TAG_INFECT)));
      if (u < p) {
        s = 1;
        d = 0;
      }
    }
  } else if (s == 1) {
    d = d + 1;
    if (d >= recovery) s = 2;
  }
  st_wr[i] = s;
  d_wr[i] = d;
}

double *ptab_address() {
  int dev = 0;
  VG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) fail(VG_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mutex);
  if (!g_ptab_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sir_ptab);
    if (e != cudaSuccess || !p)
      fail(VG_ERR_CUDA, std::string("cudaGetSymbolAddress of the SIR table failed: ") +
                            cudaGetErrorString(e));
    g_ptab_addr[dev] = (double *)p;
  }
  return g_ptab_addr[dev];
}

}  // namespace

void set_last_error(const std::string &m);

}  // namespace vg

using namespace vg;

extern "C" int vg_sir_step_noalloc(const uint32_t *row_ptr, const uint32_t *src,
                                   const uint8_t *state_in, const int32_t *days_in,
                                   uint8_t *state_out, int32_t *days_out, uint64_t n,
                                   uint32_t max_in_degree, double beta, int32_t recovery,
                                   uint64_t seed, uint32_t step, void *stream) {
  try {
    if (max_in_degree > (uint32_t)NOALLOC_MAX_DEGREE)
      fail(VG_ERR_ARG, "vg_sir_step_noalloc: max_in_degree " + std::to_string(max_in_degree) +
                           " exceeds the fixed table of " +
                           std::to_string(NOALLOC_MAX_DEGREE) + " (use apply! with \"sir\")");
    if (n == 0) return VG_OK;
    if (!row_ptr || !state_in || !days_in || !state_out || !days_out || (!src && max_in_degree))
      fail(VG_ERR_ARG, "vg_sir_step_noalloc: null buffer");
    cudaStream_t st = (cudaStream_t)stream;
    double *tab = ptab_address();
    k_fill_ptab<<<1, 1, 0, st>>>(tab, max_in_degree, beta);
    VG_CUDA(cudaGetLastError());
    k_sir_noalloc<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        row_ptr, src, state_in, days_in, state_out, days_out, n, tab, max_in_degree, beta, seed,
        step, recovery);
    VG_CUDA(cudaGetLastError());
    return VG_OK;
  } catch (const Error &e) {
    set_last_error(e.msg);
    return e.code;
  }
}
