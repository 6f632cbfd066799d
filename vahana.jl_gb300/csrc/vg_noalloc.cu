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
// Set-up: the first call in a CUDA context (the device's primary context,
// or whichever context the caller made current) looks up the array's device
// address in that context (cudaGetSymbolAddress) once and caches it under
// the context's unique id; a context that is destroyed and created again
// gets a new id and a new look-up.  Make the first call in a context before
// any stream capture.
#include <cuda.h>

#include <mutex>
#include <unordered_map>

#include "vg_internal.h"
#include "vg_philox.cuh"

namespace vg {
namespace {

constexpr int NOALLOC_MAX_DEGREE = 4095;  // largest in-degree the table covers

static __device__ __align__(256) double g_sir_ptab[NOALLOC_MAX_DEGREE + 1];

std::unordered_map<unsigned long long, double *> g_ptab_addr;  // context id -> address
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

// the unique id of the calling thread's current context (0 when none is
// current yet), through the driver's entry points: the library links the
// CUDA runtime only
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    VG_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                             &q1));
    VG_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      fail(VG_ERR_CUDA, "cuCtxGetCurrent / cuCtxGetId are not available from the driver");
    get_current = (GetCurrent)f1;
    get_id = (GetId)f2;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) fail(VG_ERR_CUDA, "cuCtxGetId failed");
  return id;
}

double *symbol_address() {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_sir_ptab);
  if (e != cudaSuccess || !p)
    fail(VG_ERR_CUDA, std::string("cudaGetSymbolAddress of the SIR table failed: ") +
                          cudaGetErrorString(e));
  return (double *)p;
}

double *ptab_address() {
  std::lock_guard<std::mutex> lk(g_setup_mutex);
  unsigned long long ctx = current_context_id();
  if (ctx) {
    auto it = g_ptab_addr.find(ctx);
    if (it != g_ptab_addr.end()) return it->second;
  }
  // the look-up also makes the device's primary context current when the
  // thread has no context yet
  double *p = symbol_address();
  if (!ctx) ctx = current_context_id();
  if (!ctx) fail(VG_ERR_CUDA, "no current CUDA context after the symbol look-up");
  g_ptab_addr[ctx] = p;
  return p;
}

// [a, a + na) and [b, b + nb) share a byte
bool overlap(const void *a, uint64_t na, const void *b, uint64_t nb) {
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
  return x < y + nb && y < x + na;
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
    // the step reads every agent's old state while it writes the new ones:
    // an output that shares memory with an input would be read half-updated
    if (overlap(state_out, n, state_in, n) || overlap(state_out, n, days_in, 4 * n) ||
        overlap(days_out, 4 * n, state_in, n) || overlap(days_out, 4 * n, days_in, 4 * n) ||
        overlap(state_out, n, days_out, 4 * n))
      fail(VG_ERR_ARG, "vg_sir_step_noalloc: the output buffers must not overlap the input "
                       "buffers or each other (no in-place step)");
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
