/*
 * ORACLE -- test infrastructure only.  A CPU restatement of Vahana.jl's
 * apply! for the three test models, used by tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg as the checker.  Nothing in the product
 * links or calls this file.
 *
 * Parity pinning: the reference publishes no golden vectors for these
 * models (it has no RNG and no such models).  This restatement is pinned by
 * (a) Philox4x32-10 checked against cuRAND's host generator, (b) the
 * reference's own integer known-answer tests, run through the generic
 * oracle (oracle/vahana_ref.py) and (c) agreement of this file with that
 * generic oracle on small graphs.
 *
 * What it restates:
 *   - per-target edge containers filled by add_edge! in call order
 *     (src/EdgeMethods.jl:478-522: push! onto the target's vector), built
 *     here from the record arrays with a sequential stable counting sort;
 *   - the sweep of transition_with_read! (src/AgentMethods.jl:193-207) with
 *     the write into a separate buffer (transition_with_write!, :159-181);
 *   - neighbour folds as sequential left folds in container order.
 * Floating point: compile with -ffp-contract=off; every product and sum is
 * rounded separately, in the order written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SHIFT_TYPE 56
#define NR_MASK ((1ull << 36) - 1)

/* ---- Philox4x32-10 (Salmon et al., SC'11), restated independently ------ */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void or_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint64_t seed,
               uint32_t *out) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  memcpy(out, c, 16);
}

static void draw(uint64_t seed, uint64_t nr, uint32_t step, uint32_t tag, uint32_t out[4]) {
  out[0] = (uint32_t)nr;
  out[1] = (uint32_t)(nr >> 32);
  out[2] = step;
  out[3] = tag;
  philox(out, (uint32_t)seed, (uint32_t)(seed >> 32));
}

static double unit(const uint32_t o[4]) {
  uint64_t u = ((uint64_t)o[1] << 32) | o[0];
  return (double)(u >> 11) * (1.0 / 9007199254740992.0);
}

enum { TAG_INIT = 1, TAG_EDGE = 2, TAG_INFECT = 3, TAG_MOVE = 4 };

/* ---- containers: per-target in-edges in add_edge! call order ----------- */
/* rowptr[n+1], src[E] (source agent_nr - 1), rec[E] (record index: the
 * position of the edge in the call sequence, to fetch its payload).
 * Targets are agent numbers 1..n of one type. */
int or_build_inedges(int64_t n, int64_t E, const uint64_t *from, const uint64_t *to,
                     uint64_t *rowptr, uint32_t *src, uint64_t *rec) {
  memset(rowptr, 0, (size_t)(n + 1) * sizeof(uint64_t));
  for (int64_t e = 0; e < E; e++) {
    uint64_t t = to[e] & NR_MASK;
    if (t < 1 || (int64_t)t > n) return 1;
    rowptr[t]++;
  }
  for (int64_t i = 0; i < n; i++) rowptr[i + 1] += rowptr[i];
  uint64_t *fill = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
  if (!fill) return 2;
  memcpy(fill, rowptr, (size_t)n * sizeof(uint64_t));
  for (int64_t e = 0; e < E; e++) { /* push! in call order */
    uint64_t t = (to[e] & NR_MASK) - 1;
    uint64_t k = fill[t]++;
    src[k] = (uint32_t)((from[e] & NR_MASK) - 1);
    rec[k] = (uint64_t)e;
  }
  free(fill);
  return 0;
}

/* ---- SIR ---------------------------------------------------------------- */
/* Person{state::UInt8 (0 S, 1 I, 2 R), days::Int32}.  S with k infected
 * in-neighbours: p = 1 - (1 - beta)^k by an explicit multiply loop, infected
 * when unit(Philox(seed, nr, step, TAG_INFECT)) < p (days = 0); I: days += 1,
 * R when days >= recovery. */
void or_sir_step(int64_t n, const uint64_t *rowptr, const uint32_t *src,
                 const uint8_t *st, const int32_t *days, uint8_t *st_o, int32_t *days_o,
                 double beta, int32_t recovery, uint64_t seed, uint32_t step, int nthreads) {
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nthreads)
  for (int64_t i = 0; i < n; i++) {
    uint8_t s = st[i];
    int32_t d = days[i];
    if (s == 0) {
      uint32_t k = 0;
      for (uint64_t q = rowptr[i]; q < rowptr[i + 1]; q++) k += st[src[q]] == 1;
      if (k > 0) {
        double om = 1.0 - beta, pw = 1.0;
        for (uint32_t j = 0; j < k; j++) pw = pw * om;
        double p = 1.0 - pw;
        uint32_t o[4];
        draw(seed, (uint64_t)i + 1, step, TAG_INFECT, o);
        if (unit(o) < p) {
          s = 1;
          d = 0;
        }
      }
    } else if (s == 1) {
      d = d + 1;
      if (d >= recovery) s = 2;
    }
    st_o[i] = s;
    days_o[i] = d;
  }
}

/* ---- bounded confidence -------------------------------------------------- */
/* x' = a x + b (swx / sw) over the in-neighbours with |x_j - x| < eps, in
 * container order; x' = x when none qualifies.  w holds the edge weights in
 * container order. */
void or_opinion_step(int64_t n, const uint64_t *rowptr, const uint32_t *src, const double *w,
                     const double *x, double *xo, double eps, double a, double b,
                     int nthreads) {
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
  for (int64_t i = 0; i < n; i++) {
    double xi = x[i], sw = 0.0, swx = 0.0;
    int64_t cnt = 0;
    for (uint64_t q = rowptr[i]; q < rowptr[i + 1]; q++) {
      double xj = x[src[q]];
      double d = xj - xi;
      if (fabs(d) < eps) {
        double p = w[q] * xj;
        sw = sw + w[q];
        swx = swx + p;
        cnt++;
      }
    }
    if (cnt) {
      double m = swx / sw;
      double l = a * xi;
      double r = b * m;
      xo[i] = l + r;
    } else {
      xo[i] = xi;
    }
  }
}

/* ---- Life B3/S23 on a 2-D raster (column-major, first index fastest:
 * cell (x, y) 1-based has linear index (x-1) + (y-1) W), Moore
 * neighbourhood as connect_raster_neighbors! builds it (src/Raster.jl:82-167):
 * periodic wraps (mod1), otherwise positions outside the raster are dropped
 * (src/Raster.jl:479-499) ------------------------------------------------ */
void or_life_step_p(int64_t W, int64_t H, int periodic, const uint8_t *a, uint8_t *o,
                    int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t y = 0; y < H; y++) {
    for (int64_t x = 0; x < W; x++) {
      int cnt = 0;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          if (!dx && !dy) continue;
          int64_t xx = x + dx, yy = y + dy;
          if (xx < 0 || xx >= W || yy < 0 || yy >= H) {
            if (!periodic) continue;
            xx = (xx + W) % W;
            yy = (yy + H) % H;
          }
          cnt += a[yy * W + xx];
        }
      uint8_t al = a[y * W + x];
      o[y * W + x] = (cnt == 3 || (al && cnt == 2)) ? 1 : 0;
    }
  }
}

void or_life_step(int64_t W, int64_t H, const uint8_t *a, uint8_t *o, int nthreads) {
  or_life_step_p(W, H, 1, a, o, nthreads);
}

/* ---- walkers: one Moore offset (stencil order, first dimension fastest,
 * centre removed) drawn by multiply-high of Philox(seed, nr, step,
 * TAG_MOVE)[0] into 8, then mod1 wrap; cell_out[i] is the 0-based linear
 * index of the new cell (the target of the walker -> cell edge). */
void or_walk_step(int64_t n, int64_t W, int64_t H, const int32_t *x, const int32_t *y,
                  int32_t *xo, int32_t *yo, int64_t *cell_out, uint64_t seed, uint32_t step,
                  int nthreads) {
  static const int dx[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  static const int dy[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t i = 0; i < n; i++) {
    uint32_t o[4];
    draw(seed, (uint64_t)i + 1, step, TAG_MOVE, o);
    uint32_t k = (uint32_t)(((uint64_t)o[0] * 8u) >> 32);
    int64_t nx = (int64_t)x[i] + dx[k], ny = (int64_t)y[i] + dy[k];
    nx = ((nx - 1) % W + W) % W + 1;
    ny = ((ny - 1) % H + H) % H + 1;
    xo[i] = (int32_t)nx;
    yo[i] = (int32_t)ny;
    cell_out[i] = (nx - 1) + (ny - 1) * W;
  }
}

/* ---- directed Chung-Lu generator (input construction, host) -----------
 * The same generator as the library's device generator, restated: expected
 * degrees w_i = min(c i^(-1/(gamma-1)), wmax) with c found by bisection on
 * the capped sum (mean degree `mean`), cumulative sums in index order; edge
 * e draws source and target by the smallest index whose cumulative sum
 * exceeds unit(Philox(seed, e, 0, tag)) * total and a weight (top53+1)/2^53. */
static uint64_t sample_cdf(const double *cdf, uint64_t n, double u) {
  uint64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (cdf[mid] > u) hi = mid; else lo = mid + 1;
  }
  return lo;
}

int or_gen_chung_lu(uint64_t N, uint64_t E, double mean, double gamma, double wmax,
                    uint64_t seed, int type_nr, uint64_t *from, uint64_t *to, double *w,
                    int nthreads) {
  double *r = (double *)malloc(N * sizeof(double));
  double *suffix = (double *)malloc((N + 1) * sizeof(double));
  double *cdf = (double *)malloc(N * sizeof(double));
  if (!r || !suffix || !cdf) return 1;
  double ex = -1.0 / (gamma - 1.0);
  for (uint64_t i = 0; i < N; i++) r[i] = pow((double)(i + 1), ex);
  suffix[N] = 0.0;
  for (uint64_t i = N; i-- > 0;) suffix[i] = suffix[i + 1] + r[i];
  double target = mean * (double)N, lo = 0.0, hi = wmax / r[N - 1];
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    uint64_t a = 0, b = N;
    while (a < b) {
      uint64_t m = (a + b) / 2;
      if (mid * r[m] >= wmax) a = m + 1; else b = m;
    }
    double sum = wmax * (double)a + mid * suffix[a];
    if (sum < target) lo = mid; else hi = mid;
  }
  double c = 0.5 * (lo + hi), acc = 0.0;
  for (uint64_t i = 0; i < N; i++) {
    double wi = c * r[i];
    if (wi > wmax) wi = wmax;
    acc += wi;
    cdf[i] = acc;
  }
  uint64_t tb = (uint64_t)type_nr << SHIFT_TYPE;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t e = 0; e < (int64_t)E; e++) {
    uint32_t o[4];
    draw(seed, (uint64_t)e, 0, 5, o);
    uint64_t s = sample_cdf(cdf, N, unit(o) * acc);
    draw(seed, (uint64_t)e, 0, 6, o);
    uint64_t d = sample_cdf(cdf, N, unit(o) * acc);
    from[e] = tb | (s + 1);
    to[e] = tb | (d + 1);
    if (w) {
      draw(seed, (uint64_t)e, 0, 7, o);
      uint64_t u = ((uint64_t)o[1] << 32) | o[0];
      w[e] = (double)((u >> 11) + 1) * (1.0 / 9007199254740992.0);
    }
  }
  free(r);
  free(suffix);
  free(cdf);
  return 0;
}

/* uniform out-edges: agent i adds k edges to t uniform in [1, N], t != i */
void or_gen_uniform_out(uint64_t N, uint32_t k, uint64_t seed, int type_nr, uint64_t *from,
                        uint64_t *to) {
  uint64_t tb = (uint64_t)type_nr << SHIFT_TYPE;
  for (uint64_t i = 1; i <= N; i++)
    for (uint32_t j = 1; j <= k; j++) {
      uint32_t o[4];
      draw(seed, i, j, TAG_EDGE, o);
      uint64_t t = (((uint64_t)o[0] * (uint64_t)(N - 1)) >> 32) + 1;
      if (t >= i) t += 1;
      uint64_t r = (i - 1) * k + (j - 1);
      from[r] = tb | i;
      to[r] = tb | t;
    }
}
