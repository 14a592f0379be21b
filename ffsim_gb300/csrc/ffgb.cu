// Host orchestration and the C ABI (include/ffsim_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <initializer_list>
#include <vector>

#include "../../include/ffsim_gb300.h"
#include "common.h"
#include "plan.h"
#include "diag.cuh"

namespace ffgb {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static std::atomic<long long> g_allocs{0};
void count_alloc() { g_allocs.fetch_add(1, std::memory_order_relaxed); }

static long long binom_h(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

// the complex64 or complex128 instantiation of a templated call
#define FFGB_DISPATCH(dtype, call_f, call_d) \
  ((dtype) == FFGB_C64 ? (call_f) : (call_d))

// ---------------------------------------------------------------------------
// per-device occupation-string tables
// ---------------------------------------------------------------------------
static std::mutex g_mu;
static std::map<std::tuple<int, int, int>, unsigned*> g_strings;

static int device_strings(int norb, int nocc, const unsigned** out) {
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_tuple(dev, norb, nocc);
  auto it = g_strings.find(key);
  if (it != g_strings.end()) {
    *out = it->second;
    return FFGB_OK;
  }
  const long long n = binom_h(norb, nocc);
  std::vector<unsigned> h((size_t)std::max<long long>(n, 1), 0u);
  if (nocc == 0) {
    h[0] = 0u;
  } else {
    unsigned x = (nocc >= 32) ? 0xffffffffu : ((1u << nocc) - 1u);
    for (long long a = 0; a < n; ++a) {
      h[(size_t)a] = x;
      // next integer with the same popcount (ascending order)
      unsigned c = x & (0u - x), r = x + c;
      x = (((r ^ x) >> 2) / c) | r;
    }
  }
  unsigned* d = nullptr;
  FFGB_CUDA(cudaMalloc(&d, h.size() * sizeof(unsigned)));
  count_alloc();
  FFGB_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  g_strings[key] = d;
  *out = d;
  return FFGB_OK;
}

// SM count of the current device, looked up once per device ordinal.
static int num_sms() {
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  n = n > 0 ? n : 132;
  if (dev >= 0 && dev < 64) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

// ---------------------------------------------------------------------------
// scratch carving
// ---------------------------------------------------------------------------
struct Scratch {
  char* base;
  size_t bytes, off = 0;
  Scratch(void* b, size_t n) : base((char*)b), bytes(n) {}
  void* take(size_t n) {
    size_t o = (off + 255) & ~(size_t)255;
    if (base == nullptr || o + n > bytes) return nullptr;
    off = o + n;
    return base + o;
  }
};

// column table (16 B/string), partial sums (8 B/row) and up to four
// string-phase tables (8 B/string) of the stage path, plus alignment slack
static size_t extras_bytes(int norb, int na, int nb) {
  long long da = binom_h(norb, na), db = nb >= 0 ? binom_h(norb, nb) : 1;
  long long m = std::max<long long>(std::max(da, db), 1);
  return (size_t)m * 16 + (size_t)m * 8 + (size_t)m * 32 + (size_t)m * 8 +
         (size_t)stage_expect_partials(m, m) * 8 + 65536;
}

// ---------------------------------------------------------------------------
// diagonal operator description (host)
// ---------------------------------------------------------------------------
struct DiagSpec {
  int mode = DIAG_NONE;
  int zrep = 0;
  double row_same[FFGB_MAXN][FFGB_MAXN];
  double col_same[FFGB_MAXN][FFGB_MAXN];
  double cross[FFGB_MAXN][FFGB_MAXN];
  DiagSpec() {
    std::memset(row_same, 0, sizeof(row_same));
    std::memset(col_same, 0, sizeof(col_same));
    std::memset(cross, 0, sizeof(cross));
  }
  DiagSpec transposed() const {
    DiagSpec d;
    d.mode = mode;
    d.zrep = zrep;
    std::memcpy(d.row_same, col_same, sizeof(row_same));
    std::memcpy(d.col_same, row_same, sizeof(col_same));
    for (int i = 0; i < FFGB_MAXN; ++i)
      for (int l = 0; l < FFGB_MAXN; ++l) d.cross[i][l] = cross[l][i];
    return d;
  }
};

// Diagonal Coulomb operator sum J^{st}_ij n_is n_jt / 2 (num rep) or the
// Z-rep form, scaled by `scale`; rows = alpha, columns = beta.
static SameTable same_table(const double (&m)[FFGB_MAXN][FFGB_MAXN]) {
  SameTable t;
  std::memcpy(t.v, m, sizeof(t.v));
  return t;
}

static DiagSpec diag_coulomb_spec(int norb, const double* aa, const double* ab, const double* bb,
                                  int zrep, double scale, int mode) {
  DiagSpec d;
  d.mode = mode;
  d.zrep = zrep;
  const double f = zrep ? 0.25 * scale : scale;
  for (int i = 0; i < norb; ++i)
    for (int j = i; j < norb; ++j) {
      double w = (i == j) ? (zrep ? 0.0 : 0.5) : 1.0;
      if (aa) d.row_same[i][j] = f * w * aa[i * norb + j];
      if (bb) d.col_same[i][j] = f * w * bb[i * norb + j];
    }
  if (ab)
    for (int i = 0; i < norb; ++i)
      for (int j = 0; j < norb; ++j) d.cross[i][j] = f * ab[i * norb + j];
  return d;
}

static DiagSpec one_body_spec(int norb, const double* ca, const double* cb, double scale, int mode) {
  DiagSpec d;
  d.mode = mode;
  for (int i = 0; i < norb; ++i) {
    if (ca) d.row_same[i][i] = scale * ca[i];
    if (cb) d.col_same[i][i] = scale * cb[i];
  }
  return d;
}

static void add_spec(DiagSpec& d, const DiagSpec& e) {
  for (int i = 0; i < FFGB_MAXN; ++i)
    for (int j = 0; j < FFGB_MAXN; ++j) {
      d.row_same[i][j] += e.row_same[i][j];
      d.col_same[i][j] += e.col_same[i][j];
      d.cross[i][j] += e.cross[i][j];
    }
}

// ---------------------------------------------------------------------------
// one pass of the sector kernel
// ---------------------------------------------------------------------------
template <typename T>
struct PassArgs {
  const SectorPlan* plan = nullptr;  // plan of the rotated sector (null = identity)
  int norb = 0, rot_nocc = 0, row_nocc = 0;
  long long n_rows = 1;
  const void* in = nullptr;
  void* out = nullptr;
  int out_op = OUT_STORE, layout = LAYOUT_SAME;
  double alpha = 1.0;
  const DiagSpec* diag = nullptr;
  bool apply_dphase = true;
  bool comp = false;           // compensated window coefficients (complex64)
  double* partials = nullptr;  // EXPECT
  int* n_ctas = nullptr;
  // occupation strings supplied by the caller (null: the shared per-shape cache)
  const unsigned* col_strings = nullptr;
  const unsigned* row_strings = nullptr;
};

template <typename T>
static int dispatch_sector(int nw, const SectorParams<T>& P, long long grid, int block, int smem,
                           cudaStream_t st, int* grid_out) {
  if constexpr (sizeof(T) == 8) {
    return launch_sector<T, 0>(P, grid, block, smem, st, grid_out);
  } else {
    switch (nw) {
      case 0: return launch_sector<T, 0>(P, grid, block, smem, st, grid_out);
      case 1: return launch_sector<T, 1>(P, grid, block, smem, st, grid_out);
      case 2: return launch_sector<T, 2>(P, grid, block, smem, st, grid_out);
      case 3: return launch_sector<T, 3>(P, grid, block, smem, st, grid_out);
      case 4: return launch_sector<T, 4>(P, grid, block, smem, st, grid_out);
      case 5: return launch_sector<T, 5>(P, grid, block, smem, st, grid_out);
      case 6: return launch_sector<T, 6>(P, grid, block, smem, st, grid_out);
      case 7: return launch_sector<T, 7>(P, grid, block, smem, st, grid_out);
      case 8: return launch_sector<T, 8>(P, grid, block, smem, st, grid_out);
      case 9: return launch_sector<T, 9>(P, grid, block, smem, st, grid_out);
      case 10: return launch_sector<T, 10>(P, grid, block, smem, st, grid_out);
      case 11: return launch_sector<T, 11>(P, grid, block, smem, st, grid_out);
      case 12: return launch_sector<T, 12>(P, grid, block, smem, st, grid_out);
      case 13: return launch_sector<T, 13>(P, grid, block, smem, st, grid_out);
      case 14: return launch_sector<T, 14>(P, grid, block, smem, st, grid_out);
      case 15: return launch_sector<T, 15>(P, grid, block, smem, st, grid_out);
      case 16: return launch_sector<T, 16>(P, grid, block, smem, st, grid_out);
      default: return fail(FFGB_ERR_UNSUPPORTED, "no window kernel for this norb");
    }
  }
}

template <typename T>
static int run_pass(const PassArgs<T>& A, Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const int norb = A.norb;
  if (norb > FFGB_MAXN) return fail(FFGB_ERR_UNSUPPORTED, "norb > 18 is not supported");
  const long long dim_ll = binom_h(norb, A.rot_nocc);
  if (dim_ll <= 0 || A.n_rows <= 0) return FFGB_OK;
  // scratch taken by this pass (column table) is free again once it is queued
  struct Restore {
    Scratch& s;
    size_t off;
    ~Restore() { s.off = off; }
  } restore{scr, scr.off};
  const int dim = (int)dim_ll;
  auto P = std::make_unique<SectorParams<T>>();
  std::memset(P.get(), 0, sizeof(SectorParams<T>));
  P->norb = norb;
  P->nocc = A.rot_nocc;
  P->dim = dim;
  P->kind = KIND_IDENTITY;
  int nw = 0;
  if (A.plan && A.plan->kind != PLAN_IDENTITY) {
    const SectorPlan& pl = *A.plan;
    if (pl.kind == PLAN_CSD && pl.b1.empty())
      return fail(FFGB_ERR_UNSUPPORTED, "nested cosine-sine plans run on the stage kernels only");
    P->kind = pl.kind;
    P->h = pl.h;
    if (pl.kind == PLAN_TRIANGLE) {
      P->n_tri = (int)pl.tri.size();
      for (size_t g = 0; g < pl.tri.size(); ++g) {
        P->tri[3 * g] = (T)pl.tri[g].c;
        P->tri[3 * g + 1] = (T)pl.tri[g].s.real();
        P->tri[3 * g + 2] = (T)pl.tri[g].s.imag();
        P->tri_l[g] = (signed char)pl.tri_l[g];
      }
    } else {
      P->comp = A.comp ? 1 : 0;
      auto lo = [](double x) { return (T)(x - (double)(T)x); };
      auto put = [&](int w, const std::vector<Givens>& v) {
        for (size_t g = 0; g < v.size(); ++g) {
          P->win[w][3 * g] = (T)v[g].c;
          P->win[w][3 * g + 1] = (T)v[g].s.real();
          P->win[w][3 * g + 2] = (T)v[g].s.imag();
          P->win_lo[w][3 * g] = lo(v[g].c);
          P->win_lo[w][3 * g + 1] = lo(v[g].s.real());
          P->win_lo[w][3 * g + 2] = lo(v[g].s.imag());
        }
      };
      if (pl.kind == PLAN_FULL) {
        put(0, pl.tri);
      } else {
        put(0, pl.b1);
        put(1, pl.b2);
        put(2, pl.a1);
        put(3, pl.a2);
        for (size_t i = 0; i < pl.cs.size(); ++i) {
          const Pair2& p = pl.cs[i];
          T* c = P->cs[i];
          T* cl = P->cs_lo[i];
          const double vals[8] = {p.g00.real(), p.g00.imag(), p.g01.real(), p.g01.imag(),
                                  p.g10.real(), p.g10.imag(), p.g11.real(), p.g11.imag()};
          for (int q = 0; q < 8; ++q) {
            c[q] = (T)vals[q];
            cl[q] = lo(vals[q]);
          }
        }
      }
      nw = norb;
    }
    if (A.apply_dphase) {
      bool trivial = true;
      for (int i = 0; i < norb; ++i) {
        const cd di = pl.kind == PLAN_CSD ? pl.csd_diag[i] : pl.diag[i];
        P->dphase[i][0] = (T)di.real();
        P->dphase[i][1] = (T)di.imag();
        if (std::abs(di - cd(1.0)) > 1e-15) trivial = false;
      }
      P->has_dphase = trivial ? 0 : 1;
    }
  }
  if (sizeof(T) == 8 && nw != 0) return fail(FFGB_ERR_ARG, "window plan requested for complex128");
  const int diag_mode = A.diag ? A.diag->mode : DIAG_NONE;
  P->n_rows = A.n_rows;
  P->in = A.in;
  P->out = A.out;
  P->out_op = A.out_op;
  P->layout = A.layout;
  P->alpha_re = (T)A.alpha;
  P->alpha_im = (T)0;
  P->diag_mode = diag_mode;
  P->chunk_bits = (diag_mode == DIAG_COEF && norb > 8) ? 8 : 4;
  const bool need_col = P->has_dphase || diag_mode != DIAG_NONE;
  if (need_col) {
    const unsigned* cs = A.col_strings;
    if (!cs) FFGB_TRY(device_strings(norb, A.rot_nocc, &cs));
    P->col_strings = cs;
  }
  if (diag_mode != DIAG_NONE) {
    const unsigned* rs = A.row_strings;
    if (!rs) FFGB_TRY(device_strings(norb, A.row_nocc, &rs));
    P->row_strings = rs;
    P->row_norb = norb;
    P->row_nocc = A.row_nocc;
    P->zrep = A.diag->zrep;
    std::memcpy(P->rsame, A.diag->row_same, sizeof(P->rsame));
    std::memcpy(P->cross, A.diag->cross, sizeof(P->cross));
    bool col_nonzero = false;
    for (int i = 0; i < FFGB_MAXN && !col_nonzero; ++i)
      for (int j = 0; j < FFGB_MAXN; ++j)
        if (A.diag->col_same[i][j] != 0.0) col_nonzero = true;
    if (col_nonzero) {
      void* tab = scr.take((size_t)dim * sizeof(C));
      if (!tab) return fail(FFGB_ERR_OOM, "scratch too small for the column table");
      col_table_kernel<T><<<(dim + 255) / 256, 256, 0, st>>>(P->col_strings, dim, norb, P->zrep,
                                                             diag_mode, same_table(A.diag->col_same), tab);
      count_launch();
      FFGB_CUDA(cudaGetLastError());
      P->col_table = tab;
    }
  }
  // rows per CTA
  const int block = sector_threads(nw);
  const size_t row_bytes = (size_t)dim * sizeof(C);
  const Layout L0 = make_layout(sizeof(T), 0, dim, norb, P->chunk_bits, P->has_dphase, diag_mode, P->kind, P->comp);
  const long long budget = 110 * 1024;
  long long rmax = (budget - L0.total) / (long long)row_bytes;
  if (rmax < 1) {
    if ((long long)L0.total + (long long)row_bytes > 227 * 1024)
      return fail(FFGB_ERR_UNSUPPORTED, "a sector row does not fit in shared memory");
    rmax = 1;
  }
  const long long want = std::max<long long>(1, (A.n_rows + 2LL * num_sms() - 1) / (2LL * num_sms()));
  int R = (int)std::min<long long>(std::min<long long>(rmax, want), 4096);
  if (R < 1) R = 1;
  P->rows_per_cta = R;
  const Layout L = make_layout(sizeof(T), R, dim, norb, P->chunk_bits, P->has_dphase, diag_mode, P->kind, P->comp);
  const long long n_chunks = (A.n_rows + R - 1) / R;
  if (A.out_op == OUT_EXPECT) {
    if (!A.partials) return fail(FFGB_ERR_ARG, "missing partials buffer");
    P->partials = A.partials;
  }
  int grid = 0;
  FFGB_TRY(dispatch_sector<T>(nw, *P, n_chunks, block, L.total, st, &grid));
  if (A.n_ctas) *A.n_ctas = grid;
  return FFGB_OK;
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
static std::vector<cd> load_mat(const double* m, int n) {
  std::vector<cd> v((size_t)n * n);
  for (size_t i = 0; i < v.size(); ++i) v[i] = cd(m[2 * i], m[2 * i + 1]);
  return v;
}
static std::vector<cd> dagger(const std::vector<cd>& m, int n) {
  std::vector<cd> v((size_t)n * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) v[(size_t)r * n + c] = std::conj(m[(size_t)c * n + r]);
  return v;
}
// V diag(d): column j of V times d[j].
static std::vector<cd> scale_cols(const std::vector<cd>& v, const std::vector<cd>& d, int n) {
  std::vector<cd> o(v);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) o[(size_t)r * n + c] *= d[c];
  return o;
}

static std::vector<cd> matmul(const std::vector<cd>& a, const std::vector<cd>& b, int n) {
  std::vector<cd> v((size_t)n * n, cd(0));
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k) {
      cd x = a[(size_t)r * n + k];
      for (int c = 0; c < n; ++c) v[(size_t)r * n + c] += x * b[(size_t)k * n + c];
    }
  return v;
}
static std::vector<cd> eye(int n) {
  std::vector<cd> v((size_t)n * n, cd(0));
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  return v;
}

template <typename T>
static int make_plan(int norb, const std::vector<cd>& V, SectorPlan& plan) {
  const bool windows = sizeof(T) == 4 && norb <= FFGB_MAXN;
  if (!plan_sector(norb, V.data(), windows, plan)) return fail(FFGB_ERR_NUMERIC, "plan failed");
  if (plan.max_err > 1e-9) return fail(FFGB_ERR_NUMERIC, "orbital rotation is not unitary");
  return FFGB_OK;
}

// ---------------------------------------------------------------------------
// stage-major complex64 path (cosine-sine plans, 9 <= norb <= 16)
// ---------------------------------------------------------------------------
template <typename T>
static bool staged(const SectorPlan* a, const SectorPlan* b) {
  if (sizeof(T) != 4 || (!a && !b)) return false;
  if (a && a->kind != PLAN_CSD) return false;
  if (b && b->kind != PLAN_CSD) return false;
  return true;
}

// Plans of W(U^dag) and W(U) around a diagonal operator Z.  The stage path's
// plan of U^dag = diag(d) N leaves out its final orbital phases: they commute
// with Z, and W(U) W(diag(d)) = W(U diag(d)), so the second plan is that of
// U diag(d) and no pass over the state applies d.  Returns whether both plans
// run on the stage path (otherwise pu is the plan of U itself).
template <typename T>
static int sandwich_plans(int norb, const std::vector<cd>& rot, SectorPlan& pd, SectorPlan& pu, bool* stage) {
  FFGB_TRY(make_plan<T>(norb, dagger(rot, norb), pd));
  *stage = false;
  if (staged<T>(&pd, nullptr)) {
    FFGB_TRY(make_plan<T>(norb, scale_cols(rot, pd.diag, norb), pu));
    if (staged<T>(&pu, nullptr)) {
      *stage = true;
      return FFGB_OK;
    }
  }
  return make_plan<T>(norb, rot, pu);
}

// Per-string table of a plan's final orbital phases (nullptr when they are all 1),
// complex of T.
template <typename T = float>
static int phase_table(const SectorPlan* p, int norb, int nocc, Scratch& scr, cudaStream_t st,
                       const void** out) {
  *out = nullptr;
  if (!p) return FFGB_OK;
  std::vector<double> d(2 * norb);
  bool trivial = true;
  for (int i = 0; i < norb; ++i) {
    d[2 * i] = p->diag[i].real();
    d[2 * i + 1] = p->diag[i].imag();
    if (std::abs(p->diag[i] - cd(1.0)) > 1e-15) trivial = false;
  }
  if (trivial) return FFGB_OK;
  const unsigned* strs = nullptr;
  FFGB_TRY(device_strings(norb, nocc, &strs));
  const long long dim = binom_h(norb, nocc);
  void* t = scr.take((size_t)dim * sizeof(typename CT<T>::type));
  if (!t) return fail(FFGB_ERR_OOM, "scratch too small for a string-phase table");
  FFGB_TRY(launch_string_phases<T>(strs, dim, norb, d.data(), t, st));
  *out = t;
  return FFGB_OK;
}

// Window-coefficient mode of the stage path: dithered FP32 rounding (unbiased
// per column; see win_coef).
constexpr int STAGE_MODE = 2;

// One sector's stage-major rotation (without the plan's final orbital phases)
// with an optional fused expectation on the last stage.
static int stage_sector(const void* in, void* out, int norb, int nocc, long long ld, long long ncols,
                        const SectorPlan& p, unsigned salt, cudaStream_t st, const StageExpectArgs* ex = nullptr,
                        int* ex_ctas = nullptr) {
  StageOpts o;
  o.mode = STAGE_MODE;
  o.salt = salt;
  o.expect = ex;
  o.expect_ctas = ex_ctas;
  return stage_rotate_rows(in, out, norb, nocc, ld, ncols, p, o, st);
}

// W(pa) (x) W(pb) of the state `in` (alpha rows), through `x` (same shape) and
// `tmp` (beta rows).  keep_t = false: the result is in x with alpha rows;
// keep_t = true: the result is in tmp with beta rows.  The plans' final
// orbital phases ride on the transposes (rows of the source are the sector
// just rotated).  With keep_t the beta phases are returned in *fb_pending for
// the caller to apply (null: applied here); phases = false leaves them out
// (they do not change |amplitude|^2).  `salt` decorrelates the coefficient
// dithering of different rotations.
static int staged_rotate(const void* in, void* x, void* tmp, int norb, int na, int nb,
                         const SectorPlan* pa, const SectorPlan* pb, bool phases, bool keep_t, unsigned salt,
                         Scratch& scr, cudaStream_t st, const void** fb_pending = nullptr) {
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  const void *fa = nullptr, *fb = nullptr;
  if (phases) {
    FFGB_TRY(phase_table(pa, norb, na, scr, st, &fa));
    FFGB_TRY(phase_table(pb, norb, nb, scr, st, &fb));
  }
  if (fb_pending) *fb_pending = nullptr;
  if (pa) FFGB_TRY(stage_sector(in, x, norb, na, db, db, *pa, 2 * salt, st));
  if (!pb && !keep_t) {
    if (!pa && in != x) FFGB_CUDA(cudaMemcpyAsync(x, in, (size_t)(da * db) * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    if (fa) FFGB_TRY(launch_row_scale<float>(x, da, db, fa, st));
    return FFGB_OK;
  }
  FFGB_TRY(launch_transpose<float>(pa ? x : in, tmp, da, db, fa, nullptr, st));
  if (pb) FFGB_TRY(stage_sector(tmp, tmp, norb, nb, da, da, *pb, 2 * salt + 1, st));
  if (keep_t) {
    if (fb_pending)
      *fb_pending = fb;
    else if (fb)
      FFGB_TRY(launch_row_scale<float>(tmp, db, da, fb, st));
    return FFGB_OK;
  }
  return launch_transpose<float>(tmp, x, db, da, fb, nullptr, st);
}

// complex64 plans that exist only as a stage sequence (norb 17-18) cannot
// run on the shared-memory sector kernel; a single sector vector (spinless)
// then runs the stage kernels as a one-column matrix.
static bool ops_only(const SectorPlan& p) { return p.kind == PLAN_CSD && p.b1.empty(); }

static int stage_spinless(void* vec, int norb, int nocc, const SectorPlan& p, unsigned salt, Scratch& scr,
                          cudaStream_t st) {
  const size_t mark = scr.off;
  FFGB_TRY(stage_sector(vec, vec, norb, nocc, 1, 1, p, salt, st));
  const void* f = nullptr;
  FFGB_TRY(phase_table(&p, norb, nocc, scr, st, &f));
  if (f) FFGB_TRY(launch_row_scale<float>(vec, binom_h(norb, nocc), 1, f, st));
  scr.off = mark;
  return FFGB_OK;
}

// Number-representation diagonal operators absorb orbital phases d_i of the
// column (beta) sector: exp(i arg(d_i) n_i) = d_i^(n_i).
static void fold_col_phases(DiagSpec& spec, const SectorPlan& p, int norb) {
  for (int i = 0; i < norb; ++i) spec.col_same[i][i] += std::arg(p.diag[i]);
}

// out (+)= D in for a diagonal operator D (PHASE: exp(i f), COEF: f) on a
// state whose rows are the strings with row_nocc electrons; `spec` is written
// with these rows.  Streams rows (any sector size).
template <typename T>
static int diag_rows(const void* in, void* out, int norb, int row_nocc, int col_nocc, const DiagSpec& spec,
                     bool accumulate, Scratch& scr, cudaStream_t st, const void* outer_row = nullptr,
                     const void* outer_col = nullptr, long long n_stacked = 0) {
  using C = typename CT<T>::type;
  const long long rows = binom_h(norb, row_nocc), cols = binom_h(norb, col_nocc);
  if (rows <= 0 || cols <= 0) return FFGB_OK;
  if (spec.mode != DIAG_PHASE && spec.mode != DIAG_COEF) return fail(FFGB_ERR_ARG, "diagonal mode");
  const size_t mark = scr.off;
  const unsigned *rs = nullptr, *cs = nullptr;
  FFGB_TRY(device_strings(norb, row_nocc, &rs));
  FFGB_TRY(device_strings(norb, col_nocc, &cs));
  void* tab = scr.take((size_t)cols * (spec.mode == DIAG_PHASE ? sizeof(C) : sizeof(T)));
  if (!tab) return fail(FFGB_ERR_OOM, "scratch too small for the column table");
  col_table_kernel<T><<<(unsigned)((cols + 255) / 256), 256, 0, st>>>(cs, (int)cols, norb, spec.zrep, spec.mode,
                                                                      same_table(spec.col_same), tab);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  auto A = std::make_unique<DiagRowsArgs<T>>();
  std::memset(A.get(), 0, sizeof(DiagRowsArgs<T>));
  A->in = (const C*)in;
  A->out = (C*)out;
  A->rows = rows;
  A->cols = cols;
  A->rstr = rs;
  A->cstr = cs;
  A->col_table = tab;
  std::memcpy(A->rsame, spec.row_same, sizeof(A->rsame));
  std::memcpy(A->cross, spec.cross, sizeof(A->cross));
  A->norb = norb;
  A->zrep = spec.zrep;
  A->mode = spec.mode;
  A->accumulate = accumulate ? 1 : 0;
  if (outer_row && outer_col) {
    A->outer_row = (const C*)outer_row;
    A->outer_col = (const C*)outer_col;
  }
  if (n_stacked > 0) {  // n_stacked states side by side, padded to whole column tiles
    A->col_period = stack_pad(cols);
    A->ld = n_stacked * A->col_period;
  }
  const long long grid = (rows + DIAG_ROWS_PER_CTA - 1) / DIAG_ROWS_PER_CTA;
  diag_rows_kernel<T><<<(unsigned)grid, DIAG_THREADS, 0, st>>>(*A);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  scr.off = mark;
  return FFGB_OK;
}

// ---------------------------------------------------------------------------
// complex128 states whose sector rows exceed shared memory (norb 17-18 near
// half filling): the generic network, one adjacent Givens rotation per launch
// on the whole state, then one pass with both sectors' final phases; diagonal
// operators stream rows.  FP64 CUDA-core work bounds these passes on GB300.
// ---------------------------------------------------------------------------
template <typename T>
static bool big_rows(int norb, int na, int nb) {
  if (sizeof(T) != 8) return false;
  const double lim = 215.0 * 1024.0;  // a row of the sector kernel, with its tables
  return (double)binom_h(norb, na) * 16.0 > lim || (nb >= 0 && (double)binom_h(norb, nb) * 16.0 > lim);
}

template <typename T>
static int big_rotate(void* vec, int norb, int na, int nb, const SectorPlan* pa, const SectorPlan* pb, bool phases,
                      Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const long long da = binom_h(norb, na), db = nb < 0 ? 1 : binom_h(norb, nb);
  auto sweep = [&](const SectorPlan* p, int spin, int nocc, long long dim_other) -> int {
    if (!p || p->kind == PLAN_IDENTITY) return FFGB_OK;
    if (p->kind != PLAN_TRIANGLE) return fail(FFGB_ERR_ARG, "generic network expected");
    if (nocc < 1 || nocc > norb - 1) return FFGB_OK;
    const long long total = binom_h(norb - 2, nocc - 1) * dim_other;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 4 * 152 * 8);
    for (size_t k = 0; k < p->tri.size(); ++k) {
      const Givens& g = p->tri[k];
      givens_sector_kernel<T><<<blocks, 256, 0, st>>>((C*)vec, norb, nocc, dim_other, spin, p->tri_l[k], (T)g.c,
                                                      (T)g.s.real(), (T)g.s.imag());
      count_launch();
      FFGB_CUDA(cudaGetLastError());
    }
    return FFGB_OK;
  };
  FFGB_TRY(sweep(pa, 0, na, db));
  if (nb >= 0) FFGB_TRY(sweep(pb, 1, nb, da));
  if (!phases) return FFGB_OK;
  const size_t mark = scr.off;
  const void *fa = nullptr, *fb = nullptr;
  FFGB_TRY(phase_table<T>(pa, norb, na, scr, st, &fa));
  if (nb >= 0) FFGB_TRY(phase_table<T>(pb, norb, nb, scr, st, &fb));
  if (fa || fb) {
    const long long n = da * db;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4 * 152 * 8);
    outer_scale_kernel<C><<<blocks, 256, 0, st>>>((C*)vec, da, db, (const C*)fa, (const C*)fb);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
  }
  scr.off = mark;
  return FFGB_OK;
}

// sum f |x|^2 of a COEF diagonal into dslot (device double).
template <typename T>
static int big_expect(const void* x, int norb, int na, int nb, const DiagSpec& spec, double* dslot, Scratch& scr,
                      cudaStream_t st) {
  using C = typename CT<T>::type;
  const size_t mark = scr.off;
  const long long rows = binom_h(norb, na), cols = binom_h(norb, nb);
  const unsigned *rs = nullptr, *cs = nullptr;
  FFGB_TRY(device_strings(norb, na, &rs));
  FFGB_TRY(device_strings(norb, nb, &cs));
  const long long grid = (rows + DIAG_ROWS_PER_CTA - 1) / DIAG_ROWS_PER_CTA;
  void* tab = scr.take((size_t)cols * sizeof(T));
  double* partials = (double*)scr.take(sizeof(double) * (size_t)grid);
  if (!tab || !partials) return fail(FFGB_ERR_OOM, "scratch too small for the expectation tables");
  col_table_kernel<T><<<(unsigned)((cols + 255) / 256), 256, 0, st>>>(cs, (int)cols, norb, spec.zrep, DIAG_COEF,
                                                                      same_table(spec.col_same), tab);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  auto A = std::make_unique<DiagRowsArgs<T>>();
  std::memset(A.get(), 0, sizeof(DiagRowsArgs<T>));
  A->in = (const C*)x;
  A->rows = rows;
  A->cols = cols;
  A->rstr = rs;
  A->cstr = cs;
  A->col_table = tab;
  std::memcpy(A->rsame, spec.row_same, sizeof(A->rsame));
  std::memcpy(A->cross, spec.cross, sizeof(A->cross));
  A->norb = norb;
  A->zrep = spec.zrep;
  A->mode = DIAG_COEF;
  A->partials = partials;
  diag_rows_kernel<T><<<(unsigned)grid, DIAG_THREADS, 0, st>>>(*A);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  reduce_partials_kernel<<<1, 256, 0, st>>>(partials, (int)grid, dslot, 0);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  scr.off = mark;
  return FFGB_OK;
}

// Diagonal operator on a state held with beta rows (db rows of da columns):
// in place (PHASE / COEF) or reduced into partial sums (EXPECT).  `spec` is
// written with alpha rows.
template <typename T>
static int diag_pass_t(void* t, int norb, int na, int nb, const DiagSpec& spec, int out_op, double* partials,
                       int* n_ctas, Scratch& scr, cudaStream_t st) {
  DiagSpec dt = spec.transposed();
  if (sizeof(T) == 4 && out_op == OUT_STORE) return diag_rows<T>(t, t, norb, nb, na, dt, false, scr, st);
  PassArgs<T> A;
  A.norb = norb;
  A.rot_nocc = na;
  A.row_nocc = nb;
  A.n_rows = binom_h(norb, nb);
  A.in = t;
  A.out = out_op == OUT_EXPECT ? nullptr : t;
  A.out_op = out_op;
  A.layout = LAYOUT_SAME;
  A.diag = &dt;
  A.partials = partials;
  A.n_ctas = n_ctas;
  return run_pass<T>(A, scr, st);
}

// Both sectors rotated, state (dim_a, dim_b) in `vec`; the result lands in
// `vec` (two transposing passes through `tmp`).  Optional diagonal operator
// applied in the second pass (rows = beta).
template <typename T>
static int rotate_both(void* vec, void* tmp, int norb, int na, int nb, const SectorPlan* pa,
                       const SectorPlan* pb, const DiagSpec* diag_ab, Scratch& scr,
                       cudaStream_t st, bool comp = false) {
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  PassArgs<T> A;
  A.plan = pb;
  A.norb = norb;
  A.rot_nocc = nb;
  A.row_nocc = na;
  A.n_rows = da;
  A.in = vec;
  A.out = tmp;
  A.layout = LAYOUT_T;
  A.comp = comp;
  FFGB_TRY(run_pass<T>(A, scr, st));
  DiagSpec dt;
  PassArgs<T> B;
  B.plan = pa;
  B.norb = norb;
  B.rot_nocc = na;
  B.row_nocc = nb;
  B.n_rows = db;
  B.in = tmp;
  B.out = vec;
  B.layout = LAYOUT_T;
  B.comp = comp;
  if (diag_ab) {
    dt = diag_ab->transposed();
    B.diag = &dt;
  }
  return run_pass<T>(B, scr, st);
}

// Plans of both sectors' rotations; a spin-balanced rotation (the same
// matrix for both) is planned once.
template <typename T>
static int plan_pair(int norb, const double* ma, const double* mb, SectorPlan& pa, SectorPlan& pb) {
  if (ma) FFGB_TRY(make_plan<T>(norb, load_mat(ma, norb), pa));
  if (!mb) return FFGB_OK;
  if (ma && (ma == mb || std::memcmp(ma, mb, sizeof(double) * 2 * (size_t)norb * norb) == 0)) {
    pb = pa;
    return FFGB_OK;
  }
  return make_plan<T>(norb, load_mat(mb, norb), pb);
}

template <typename T>
static int orbital_rotation_impl(void* vec, int norb, int na, int nb, const double* ma,
                                 const double* mb, Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  if (big_rows<T>(norb, na, nb)) {
    SectorPlan pa, pb;
    FFGB_TRY(plan_pair<T>(norb, ma, nb >= 0 ? mb : nullptr, pa, pb));
    return big_rotate<T>(vec, norb, na, nb, ma ? &pa : nullptr, mb && nb >= 0 ? &pb : nullptr, true, scr, st);
  }
  if (nb < 0) {  // spinless
    if (!ma) return FFGB_OK;
    SectorPlan p;
    FFGB_TRY(make_plan<T>(norb, load_mat(ma, norb), p));
    if (sizeof(T) == 4 && ops_only(p)) return stage_spinless(vec, norb, na, p, 1, scr, st);
    PassArgs<T> A;
    A.plan = &p;
    A.norb = norb;
    A.rot_nocc = na;
    A.row_nocc = 0;
    A.n_rows = 1;
    A.in = vec;
    A.out = vec;
    return run_pass<T>(A, scr, st);
  }
  SectorPlan pa, pb;
  FFGB_TRY(plan_pair<T>(norb, ma, mb, pa, pb));
  if (!ma && !mb) return FFGB_OK;
  if (!ma) {  // beta only: rows are alpha strings, in place
    if (sizeof(T) == 4 && ops_only(pb)) {
      const size_t S = (size_t)binom_h(norb, na) * binom_h(norb, nb) * sizeof(C);
      void* tmp = scr.take(S);
      if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
      return staged_rotate(vec, vec, tmp, norb, na, nb, nullptr, &pb, true, false, 1, scr, st);
    }
    PassArgs<T> A;
    A.plan = &pb;
    A.norb = norb;
    A.rot_nocc = nb;
    A.row_nocc = na;
    A.n_rows = binom_h(norb, na);
    A.in = vec;
    A.out = vec;
    return run_pass<T>(A, scr, st);
  }
  const size_t S = (size_t)binom_h(norb, na) * binom_h(norb, nb) * sizeof(C);
  void* tmp = scr.take(S);
  if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
  // Up to 12 orbitals a state is at most 6.8 MB and the time goes to launches:
  // the two transposing sector-kernel passes beat the stage path's ~40
  // launches (measured: 0.068 against 0.123 ms at norb 10, 0.145 against
  // 0.169 ms at norb 12)
  if (norb > 12 && staged<T>(&pa, mb ? &pb : nullptr))
    return staged_rotate(vec, vec, tmp, norb, na, nb, &pa, mb ? &pb : nullptr, true, false, 1, scr, st);
  return rotate_both<T>(vec, tmp, norb, na, nb, &pa, mb ? &pb : nullptr, nullptr, scr, st);
}

// Plans of U^dag and U for both sectors (rotations conjugating a diagonal
// operator); the same matrix for both sectors is planned once.
template <typename T>
static int plan_conj_pair(int norb, const double* rot_a, const double* rot_b, SectorPlan& pad, SectorPlan& pau,
                          SectorPlan& pbd, SectorPlan& pbu) {
  if (rot_a) {
    auto U = load_mat(rot_a, norb);
    FFGB_TRY(make_plan<T>(norb, dagger(U, norb), pad));
    FFGB_TRY(make_plan<T>(norb, U, pau));
  }
  if (!rot_b) return FFGB_OK;
  if (rot_a && (rot_a == rot_b || std::memcmp(rot_a, rot_b, sizeof(double) * 2 * (size_t)norb * norb) == 0)) {
    pbd = pad;
    pbu = pau;
    return FFGB_OK;
  }
  auto U = load_mat(rot_b, norb);
  FFGB_TRY(make_plan<T>(norb, dagger(U, norb), pbd));
  return make_plan<T>(norb, U, pbu);
}

// W(U) D W(U)^dag vec with D a diagonal phase operator (evolution)
template <typename T>
static int diag_evolution_impl(void* vec, int norb, int na, int nb, const DiagSpec& spec,
                               const double* rot_a, const double* rot_b, Scratch& scr,
                               cudaStream_t st) {
  using C = typename CT<T>::type;
  if (big_rows<T>(norb, na, nb)) {
    const bool rb = rot_b && nb >= 0;
    SectorPlan pad, pbd, pau, pbu;
    FFGB_TRY(plan_conj_pair<T>(norb, rot_a, rb ? rot_b : nullptr, pad, pau, pbd, pbu));
    FFGB_TRY(big_rotate<T>(vec, norb, na, nb, rot_a ? &pad : nullptr, rb ? &pbd : nullptr, true, scr, st));
    if (nb < 0) {  // spinless: one row whose columns are the strings
      DiagSpec d = spec;
      std::memcpy(d.col_same, spec.row_same, sizeof(d.col_same));
      std::memset(d.row_same, 0, sizeof(d.row_same));
      std::memset(d.cross, 0, sizeof(d.cross));
      FFGB_TRY(diag_rows<T>(vec, vec, norb, 0, na, d, false, scr, st));
    } else {
      FFGB_TRY(diag_rows<T>(vec, vec, norb, na, nb, spec, false, scr, st));
    }
    return big_rotate<T>(vec, norb, na, nb, rot_a ? &pau : nullptr, rb ? &pbu : nullptr, true, scr, st);
  }
  if (nb < 0) {  // spinless: one row
    SectorPlan pu, pd;
    if (rot_a) {
      auto U = load_mat(rot_a, norb);
      FFGB_TRY(make_plan<T>(norb, dagger(U, norb), pd));
      FFGB_TRY(make_plan<T>(norb, U, pu));
    }
    DiagSpec d = spec;
    std::memcpy(d.col_same, spec.row_same, sizeof(d.col_same));
    std::memset(d.row_same, 0, sizeof(d.row_same));
    std::memset(d.cross, 0, sizeof(d.cross));
    if (sizeof(T) == 4 && rot_a && ops_only(pd)) {
      FFGB_TRY(stage_spinless(vec, norb, na, pd, 2, scr, st));
      FFGB_TRY(diag_rows<T>(vec, vec, norb, 0, na, d, false, scr, st));
      return stage_spinless(vec, norb, na, pu, 3, scr, st);
    }
    if (sizeof(T) == 4 && !rot_a) return diag_rows<T>(vec, vec, norb, 0, na, d, false, scr, st);
    PassArgs<T> A;
    A.plan = rot_a ? &pd : nullptr;
    A.norb = norb;
    A.rot_nocc = na;
    A.row_nocc = 0;
    A.n_rows = 1;
    A.in = vec;
    A.out = vec;
    A.diag = &d;
    FFGB_TRY(run_pass<T>(A, scr, st));
    if (rot_a) {
      PassArgs<T> B = A;
      B.plan = &pu;
      B.diag = nullptr;
      FFGB_TRY(run_pass<T>(B, scr, st));
    }
    return FFGB_OK;
  }
  const long long da = binom_h(norb, na);
  if (!rot_a && !rot_b) return diag_rows<T>(vec, vec, norb, na, nb, spec, false, scr, st);
  SectorPlan pad, pbd, pau, pbu;
  FFGB_TRY(plan_conj_pair<T>(norb, rot_a, rot_b, pad, pau, pbd, pbu));
  const size_t S = (size_t)da * binom_h(norb, nb) * sizeof(C);
  void* tmp = scr.take(S);
  if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
  const SectorPlan *sad = rot_a ? &pad : nullptr, *sbd = rot_b ? &pbd : nullptr;
  if (staged<T>(sad, sbd)) {
    // W(U) D W(U)^dag: rotate into the beta-row layout, diagonal, beta back, alpha back
    const void* fbp = nullptr;
    FFGB_TRY(staged_rotate(vec, vec, tmp, norb, na, nb, sad, sbd, true, true, 2, scr, st, &fbp));
    const long long db = binom_h(norb, nb);
    if (fbp && !spec.zrep) {
      DiagSpec s2 = spec;
      fold_col_phases(s2, pbd, norb);
      FFGB_TRY(diag_pass_t<T>(tmp, norb, na, nb, s2, OUT_STORE, nullptr, nullptr, scr, st));
    } else {
      if (fbp) FFGB_TRY(launch_row_scale<float>(tmp, db, da, fbp, st));
      FFGB_TRY(diag_pass_t<T>(tmp, norb, na, nb, spec, OUT_STORE, nullptr, nullptr, scr, st));
    }
    const void *fa = nullptr, *fb = nullptr;
    FFGB_TRY(phase_table(rot_a ? &pau : nullptr, norb, na, scr, st, &fa));
    FFGB_TRY(phase_table(rot_b ? &pbu : nullptr, norb, nb, scr, st, &fb));
    if (rot_b) FFGB_TRY(stage_sector(tmp, tmp, norb, nb, da, da, pbu, 7, st));
    FFGB_TRY(launch_transpose<float>(tmp, vec, db, da, fb, nullptr, st));
    if (rot_a) FFGB_TRY(stage_sector(vec, vec, norb, na, db, db, pau, 6, st));
    if (fa) FFGB_TRY(launch_row_scale<float>(vec, da, db, fa, st));
    return FFGB_OK;
  }
  FFGB_TRY(rotate_both<T>(vec, tmp, norb, na, nb, rot_a ? &pad : nullptr, rot_b ? &pbd : nullptr,
                          &spec, scr, st));
  return rotate_both<T>(vec, tmp, norb, na, nb, rot_a ? &pau : nullptr, rot_b ? &pbu : nullptr,
                        nullptr, scr, st);
}

// out (+)= W(rot) Z W(rot)^dag vec, Z real diagonal
template <typename T>
static int rotated_matvec_impl(const void* vec, void* out, int norb, int na, int nb,
                               const DiagSpec& spec, const std::vector<cd>* rot, int accumulate,
                               Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  if (big_rows<T>(norb, na, nb)) {
    if (!rot) return diag_rows<T>(vec, out, norb, na, nb, spec, accumulate != 0, scr, st);
    SectorPlan pd, pu;
    FFGB_TRY(make_plan<T>(norb, dagger(*rot, norb), pd));
    FFGB_TRY(make_plan<T>(norb, *rot, pu));
    const size_t S = (size_t)da * db * sizeof(C);
    void* t1 = scr.take(S);
    if (!t1) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
    FFGB_CUDA(cudaMemcpyAsync(t1, vec, S, cudaMemcpyDeviceToDevice, st));
    FFGB_TRY(big_rotate<T>(t1, norb, na, nb, &pd, &pd, true, scr, st));
    FFGB_TRY(diag_rows<T>(t1, t1, norb, na, nb, spec, false, scr, st));
    FFGB_TRY(big_rotate<T>(t1, norb, na, nb, &pu, &pu, true, scr, st));
    if (accumulate) return launch_axpy<T>(t1, out, da * db, 1.0, st);
    FFGB_CUDA(cudaMemcpyAsync(out, t1, S, cudaMemcpyDeviceToDevice, st));
    return FFGB_OK;
  }
  if (!rot) return diag_rows<T>(vec, out, norb, na, nb, spec, accumulate != 0, scr, st);
  SectorPlan pd, pu;
  bool stage = false;
  FFGB_TRY(sandwich_plans<T>(norb, *rot, pd, pu, &stage));
  const size_t S = (size_t)da * db * sizeof(C);
  void* t1 = scr.take(S);
  void* t2 = scr.take(S);
  if (!t1 || !t2) return fail(FFGB_ERR_OOM, "scratch too small (needs two states)");
  if (stage) {
    // W(N) without the phases of the U^dag plan, which pu carries
    FFGB_TRY(staged_rotate(vec, t1, t2, norb, na, nb, &pd, &pd, false, true, 4, scr, st));
    FFGB_TRY(diag_pass_t<T>(t2, norb, na, nb, spec, OUT_STORE, nullptr, nullptr, scr, st));
    const void *fa = nullptr, *fb = nullptr;
    FFGB_TRY(phase_table(&pu, norb, na, scr, st, &fa));
    FFGB_TRY(phase_table(&pu, norb, nb, scr, st, &fb));
    FFGB_TRY(stage_sector(t2, t2, norb, nb, da, da, pu, 11, st));
    FFGB_TRY(launch_transpose<float>(t2, t1, db, da, fb, nullptr, st));
    if (!accumulate) {
      FFGB_TRY(stage_sector(t1, out, norb, na, db, db, pu, 10, st));
      return fa ? launch_row_scale<float>(out, da, db, fa, st) : FFGB_OK;
    }
    FFGB_TRY(stage_sector(t1, t1, norb, na, db, db, pu, 10, st));
    return launch_row_axpy<float>(t1, out, da, db, fa, st);
  }
  PassArgs<T> A;
  A.norb = norb;
  A.layout = LAYOUT_T;
  A.plan = &pd;
  A.rot_nocc = nb;
  A.row_nocc = na;
  A.n_rows = da;
  A.in = vec;
  A.out = t1;
  FFGB_TRY(run_pass<T>(A, scr, st));
  DiagSpec dt = spec.transposed();
  PassArgs<T> B = A;
  B.plan = &pd;
  B.rot_nocc = na;
  B.row_nocc = nb;
  B.n_rows = db;
  B.in = t1;
  B.out = t2;
  B.diag = &dt;
  FFGB_TRY(run_pass<T>(B, scr, st));
  A.plan = &pu;
  A.in = t2;
  A.out = t1;
  FFGB_TRY(run_pass<T>(A, scr, st));
  B.plan = &pu;
  B.in = t1;
  B.out = out;
  B.diag = nullptr;
  B.out_op = accumulate ? OUT_ACCUM : OUT_STORE;
  return run_pass<T>(B, scr, st);
}

// Tables of the fused expectation for a state held with beta rows (rows =
// beta strings, columns = alpha strings); `spec` is written with alpha rows.
static int expect_tables(int norb, int na, int nb, const DiagSpec& spec, Scratch& scr, cudaStream_t st,
                         StageExpectArgs& ex) {
  const DiagSpec dt = spec.transposed();
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  const unsigned *sa = nullptr, *sb = nullptr;
  FFGB_TRY(device_strings(norb, na, &sa));
  FFGB_TRY(device_strings(norb, nb, &sb));
  float* zrow = (float*)scr.take(sizeof(float) * (size_t)db);
  float* zcol = (float*)scr.take(sizeof(float) * (size_t)da);
  if (!zrow || !zcol) return fail(FFGB_ERR_OOM, "scratch too small for the expectation tables");
  col_table_kernel<float><<<(unsigned)((db + 255) / 256), 256, 0, st>>>(sb, (int)db, norb, dt.zrep, DIAG_COEF,
                                                                         same_table(dt.row_same), zrow);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  col_table_kernel<float><<<(unsigned)((da + 255) / 256), 256, 0, st>>>(
      sa, (int)da, norb, dt.zrep, DIAG_COEF, same_table(dt.col_same), zcol);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  ex.zrow = zrow;
  ex.zcol = zcol;
  ex.row_str = sb;
  ex.col_str = sa;
  ex.zrep = dt.zrep;
  for (int i = 0; i < FFGB_MAXN; ++i)
    for (int l = 0; l < FFGB_MAXN; ++l) ex.X[i][l] = (float)dt.cross[i][l];
  return FFGB_OK;
}

// <vec| W(V)^dag... : sum z |W(V) vec|^2 into dslot (device double)
template <typename T>
static int expectation_term(const void* vec, int norb, int na, int nb, const DiagSpec& spec,
                            const std::vector<cd>& V, void* tmp, void* tmp2, double* dslot, unsigned salt,
                            Scratch& scr, cudaStream_t st) {
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  SectorPlan pv;
  FFGB_TRY(make_plan<T>(norb, V, pv));
  const size_t mark = scr.off;
  if (big_rows<T>(norb, na, nb)) {  // |phi|^2 does not see the final orbital phases
    FFGB_CUDA(cudaMemcpyAsync(tmp, vec, (size_t)(da * db) * sizeof(typename CT<T>::type), cudaMemcpyDeviceToDevice,
                              st));
    FFGB_TRY(big_rotate<T>(tmp, norb, na, nb, &pv, &pv, false, scr, st));
    FFGB_TRY(big_expect<T>(tmp, norb, na, nb, spec, dslot, scr, st));
    scr.off = mark;
    return FFGB_OK;
  }
  if (tmp2 && staged<T>(&pv, &pv)) {
    // alpha stages into tmp, transpose to beta rows, beta stages with the
    // expectation fused into the last one (no phases: |psi|^2 does not see them)
    FFGB_TRY(stage_sector(vec, tmp, norb, na, db, db, pv, 2 * salt, st));
    FFGB_TRY(launch_transpose<float>(tmp, tmp2, da, db, nullptr, nullptr, st));
    StageExpectArgs ex;
    FFGB_TRY(expect_tables(norb, na, nb, spec, scr, st, ex));
    ex.partial_cap = stage_expect_partials(db, da);
    ex.partials = (double*)scr.take(sizeof(double) * (size_t)ex.partial_cap);
    if (!ex.partials) return fail(FFGB_ERR_OOM, "scratch too small for partial sums");
    int nct = 0;
    FFGB_TRY(stage_sector(tmp2, tmp2, norb, nb, da, da, pv, 2 * salt + 1, st, &ex, &nct));
    reduce_partials_kernel<<<1, 256, 0, st>>>(ex.partials, nct, dslot, 0);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
    scr.off = mark;
    return FFGB_OK;
  }
  PassArgs<T> A;
  A.norb = norb;
  A.layout = LAYOUT_T;
  A.plan = &pv;
  A.rot_nocc = nb;
  A.row_nocc = na;
  A.n_rows = da;
  A.in = vec;
  A.out = tmp;
  A.apply_dphase = false;  // |phi|^2 does not see the final orbital phases
  A.comp = true;           // coherent coefficient rounding would bias every term
  FFGB_TRY(run_pass<T>(A, scr, st));
  double* partials = (double*)scr.take(sizeof(double) * (size_t)std::max<long long>(db, 1));
  if (!partials) return fail(FFGB_ERR_OOM, "scratch too small for partial sums");
  DiagSpec dt = spec.transposed();
  PassArgs<T> B = A;
  B.rot_nocc = na;
  B.row_nocc = nb;
  B.n_rows = db;
  B.in = tmp;
  B.out = nullptr;
  B.out_op = OUT_EXPECT;
  B.diag = &dt;
  B.partials = partials;
  int nct = 0;
  B.n_ctas = &nct;
  FFGB_TRY(run_pass<T>(B, scr, st));
  reduce_partials_kernel<<<1, 256, 0, st>>>(partials, nct, dslot, 0);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  scr.off = mark;
  return FFGB_OK;
}

// One UCJ layer on x: both sectors rotated by the plan p, then the diagonal
// phase operator `spec` (none for the final rotation).  Compensated
// coefficients in complex64.
template <typename T>
static int ucj_layer(void* x, void* tmp, int norb, int na, int nb, const SectorPlan& p, const DiagSpec* spec,
                     unsigned salt, Scratch& scr, cudaStream_t st) {
  if (big_rows<T>(norb, na, nb)) {
    FFGB_TRY(big_rotate<T>(x, norb, na, nb, &p, &p, true, scr, st));
    return spec ? diag_rows<T>(x, x, norb, na, nb, *spec, false, scr, st) : FFGB_OK;
  }
  if (staged<T>(&p, &p)) {
    const size_t mark = scr.off;
    const void* fbp = nullptr;
    FFGB_TRY(staged_rotate(x, x, tmp, norb, na, nb, &p, &p, true, spec != nullptr, salt, scr, st, &fbp));
    if (spec) {
      DiagSpec s2 = *spec;
      if (fbp) {
        if (s2.zrep)
          FFGB_TRY(launch_row_scale<float>(tmp, binom_h(norb, nb), binom_h(norb, na), fbp, st));
        else
          fold_col_phases(s2, p, norb);
      }
      FFGB_TRY(diag_pass_t<T>(tmp, norb, na, nb, s2, OUT_STORE, nullptr, nullptr, scr, st));
      FFGB_TRY(launch_transpose<float>(tmp, x, binom_h(norb, nb), binom_h(norb, na), nullptr, nullptr, st));
    }
    scr.off = mark;
    return FFGB_OK;
  }
  return rotate_both<T>(x, tmp, norb, na, nb, &p, &p, spec, scr, st, sizeof(T) == 4);
}

// First UCJ layer from the Hartree-Fock state: W(V) |HF> is the product of
// one determinant vector per sector, amp(a, b) = det V[occ(a), :n_a] *
// det V[occ(b), :n_b], so the layer's rotation is one write pass (the
// determinants in FP64, then the diagonal phase on the outer product) instead
// of a two-sector rotation.
template <typename T>
static int slater_layer(void* x, int norb, int na, int nb, const std::vector<cd>& V, const DiagSpec& spec,
                        Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const size_t mark = scr.off;
  SlaterMat M;
  std::memset(&M, 0, sizeof(M));
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j < norb; ++j) {
      M.v[2 * (i * norb + j)] = V[(size_t)i * norb + j].real();
      M.v[2 * (i * norb + j) + 1] = V[(size_t)i * norb + j].imag();
    }
  void* vecs[2] = {nullptr, nullptr};
  const int nocc[2] = {na, nb};
  for (int sct = 0; sct < 2; ++sct) {
    const long long dim = binom_h(norb, nocc[sct]);
    const unsigned* strs = nullptr;
    FFGB_TRY(device_strings(norb, nocc[sct], &strs));
    vecs[sct] = scr.take((size_t)dim * sizeof(C));
    if (!vecs[sct]) return fail(FFGB_ERR_OOM, "scratch too small for the determinant vectors");
    slater_dets_kernel<C><<<(unsigned)((dim + 127) / 128), 128, 0, st>>>(strs, dim, norb, nocc[sct], M,
                                                                          (C*)vecs[sct]);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
  }
  FFGB_TRY(diag_rows<T>(nullptr, x, norb, na, nb, spec, false, scr, st, vecs[0], vecs[1]));
  scr.off = mark;
  return FFGB_OK;
}

// The UCJ layers of ffgb_lucj_energy on `work` (from the Hartree-Fock state
// when slater_start, the first layer then a Slater determinant; otherwise from
// the state already in `work`), with the circuit's last rotation left out:
// `basis` returns it (U_L), to be applied or merged into what follows.
static int ucj_layers(void* work, void* tmp, int dtype, int norb, int na, int nb, int n_reps, const double* ucj_dcm,
                      const double* ucj_rots, bool slater_start, Scratch& scr, cudaStream_t st,
                      std::vector<cd>& basis) {
  basis = eye(norb);
  for (int k = 0; k < n_reps; ++k) {
    std::vector<cd> U = load_mat(ucj_rots + (size_t)k * norb * norb * 2, norb);
    std::vector<cd> V = matmul(dagger(U, norb), basis, norb);
    const double* J = ucj_dcm + (size_t)k * 2 * norb * norb;
    DiagSpec spec = diag_coulomb_spec(norb, J, J + norb * norb, J, 0, 1.0, DIAG_PHASE);
    if (k == 0 && slater_start) {
      FFGB_TRY(dtype == FFGB_C64 ? slater_layer<float>(work, norb, na, nb, V, spec, scr, st)
                                 : slater_layer<double>(work, norb, na, nb, V, spec, scr, st));
      basis = U;
      continue;
    }
    SectorPlan p;
    int s = dtype == FFGB_C64 ? make_plan<float>(norb, V, p) : make_plan<double>(norb, V, p);
    if (s) return s;
    s = dtype == FFGB_C64 ? ucj_layer<float>(work, tmp, norb, na, nb, p, &spec, 20u + (unsigned)k, scr, st)
                          : ucj_layer<double>(work, tmp, norb, na, nb, p, &spec, 0, scr, st);
    if (s) return s;
    basis = U;
  }
  return FFGB_OK;
}

// DF Hamiltonian terms as (Z spec, rotation V = term basis)
struct Term {
  DiagSpec spec;
  std::vector<cd> rot;  // U (the linop is U Z U^dag)
};

static int df_terms(int norb, const double* one_body, int n_terms, const double* dcm,
                    const double* rots, int zrep, std::vector<Term>& terms) {
  terms.clear();
  if (one_body) {
    std::vector<cd> K = load_mat(one_body, norb);
    std::vector<double> w;
    std::vector<cd> vecs;
    hermitian_eigh(norb, K.data(), w, vecs);
    Term t;
    t.spec = one_body_spec(norb, w.data(), w.data(), 1.0, DIAG_COEF);
    t.rot = vecs;
    terms.push_back(std::move(t));
  }
  for (int k = 0; k < n_terms; ++k) {
    const double* J = dcm + (size_t)k * norb * norb;
    Term t;
    t.spec = diag_coulomb_spec(norb, J, J, J, zrep, 1.0, DIAG_COEF);
    t.rot = load_mat(rots + (size_t)k * norb * norb * 2, norb);
    terms.push_back(std::move(t));
  }
  return FFGB_OK;
}

// Every state has at least one amplitude, so its device buffers are never
// optional: a NULL pointer is refused here instead of reaching a kernel.
static int need_buffers(std::initializer_list<const void*> ptrs) {
  for (const void* ptr : ptrs)
    if (!ptr) return fail(FFGB_ERR_ARG, "a required buffer is NULL");
  return FFGB_OK;
}

static int check_shape(int dtype, int norb, int na, int nb) {
  if (dtype != FFGB_C64 && dtype != FFGB_C128) return fail(FFGB_ERR_DTYPE, "dtype must be complex64 or complex128");
  if (norb < 0 || norb > FFGB_MAXN) return fail(FFGB_ERR_UNSUPPORTED, "norb must be in [0, 18]");
  if (na < 0 || na > norb || nb > norb) return fail(FFGB_ERR_ARG, "invalid electron numbers");
  return FFGB_OK;
}

}  // namespace ffgb

using namespace ffgb;

template <typename T>
static int givens_impl(void* vec, int norb, int na, int nb, int spin, double c, double sr, double si,
                       int i, int j, cudaStream_t st) {
  if (std::abs(i - j) != 1) return fail(FFGB_ERR_ARG, "Target orbitals must be adjacent.");
  if (i < 0 || j < 0 || i >= norb || j >= norb) return fail(FFGB_ERR_ARG, "orbital index out of range");
  const int nocc = spin == 0 ? na : nb;
  const long long dim_other = nb < 0 ? 1 : binom_h(norb, spin == 0 ? nb : na);
  // the kernel rotates (x: lower orbital occupied, y: upper occupied) with
  // x <- c x + s y; the reference's slice1 holds strings with i occupied
  double s_re = sr, s_im = si;
  if (i > j) {  // slice1 = upper orbital occupied: s' = -conj(s)
    s_re = -sr;
    s_im = si;
  }
  const int l = std::min(i, j);
  const long long npairs = binom_h(norb - 2, nocc - 1);
  const long long total = npairs * dim_other;
  if (total <= 0) return FFGB_OK;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 8192);
  givens_sector_kernel<T><<<blocks, 256, 0, st>>>((typename CT<T>::type*)vec, norb, nocc, dim_other,
                                                  nb < 0 ? 1 : spin, l, (T)c, (T)s_re, (T)s_im);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

template <typename T>
static int df_expectation_impl(const void* vec, int norb, int na, int nb, const std::vector<Term>& terms,
                               const std::vector<cd>* pre, double constant, double* energy,
                               Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const size_t S = (size_t)binom_h(norb, na) * binom_h(norb, nb) * sizeof(C);
  void* tmp = scr.take(S);
  void* tmp2 = sizeof(T) == 4 ? scr.take(S) : nullptr;
  double* slots = (double*)scr.take(sizeof(double) * (terms.size() + 1));
  if (!tmp || !slots || (sizeof(T) == 4 && !tmp2)) return fail(FFGB_ERR_OOM, "scratch too small (needs two states)");
  for (size_t k = 0; k < terms.size(); ++k) {
    std::vector<cd> V = dagger(terms[k].rot, norb);
    if (pre) V = matmul(V, *pre, norb);
    FFGB_TRY(expectation_term<T>(vec, norb, na, nb, terms[k].spec, V, tmp, tmp2, slots + k,
                                 100u + (unsigned)k, scr, st));
  }
  std::vector<double> h(terms.size() + 1, 0.0);
  if (!terms.empty())
    FFGB_CUDA(cudaMemcpyAsync(h.data(), slots, sizeof(double) * terms.size(), cudaMemcpyDeviceToHost, st));
  FFGB_CUDA(cudaStreamSynchronize(st));
  double e = constant;
  for (size_t k = 0; k < terms.size(); ++k) e += h[k];
  *energy = e;
  return FFGB_OK;
}

// ---------------------------------------------------------------------------
// batches: n states of one shape under one Hamiltonian
// ---------------------------------------------------------------------------
// The Hamiltonian's terms are shared by every state of a batch, so each term
// runs once over all of them: the states sit side by side along the columns
// ("stacked"), alpha rows [dim_a][n * pad_b] or beta rows [dim_b][n * pad_a],
// each state padded with zero columns to whole column tiles.  The stage
// kernels act on every column independently, so one launch per stage covers
// the batch; zero columns stay zero.  The coefficient dithering of a column
// is that of its column within its state and each column tile belongs to one
// state, so a state's result is the same as when it runs alone (up to the
// order of the final FP64 sums).
struct Stack {
  long long n, da, db, pa, pb;
  size_t ybytes() const { return (size_t)(da * n * pb) * sizeof(float2); }  // alpha rows
  size_t tbytes() const { return (size_t)(db * n * pa) * sizeof(float2); }  // beta rows
};

static StageOpts stack_opts(unsigned salt, long long period) {
  StageOpts o;
  o.mode = STAGE_MODE;
  o.salt = salt;
  o.col_period = period;
  return o;
}

// <phi_b| Z |phi_b> for every state b of the stack Y (alpha rows, not
// modified), phi_b = W(V) psi_b, into slots[0..n) (device).  Y1 and T are
// stacked scratch; T's padding columns must be zero.
static int stack_expectation_term(const void* Y, void* Y1, void* T, const Stack& d, int norb, int na, int nb,
                                  const DiagSpec& spec, const SectorPlan& pv, double* slots, unsigned salt,
                                  Scratch& scr, cudaStream_t st) {
  const size_t mark = scr.off;
  FFGB_TRY(stage_rotate_rows(Y, Y1, norb, na, d.n * d.pb, d.n * d.pb, pv, stack_opts(2 * salt, d.pb), st));
  FFGB_TRY(launch_transpose_stacked<float>(Y1, T, d.da, d.db, d.n, d.pb, d.pa, nullptr, st));
  StageExpectArgs ex;
  FFGB_TRY(expect_tables(norb, na, nb, spec, scr, st, ex));
  ex.col_period = d.pa;
  ex.col_valid = d.da;
  ex.partial_cap = stage_expect_partials(d.db, d.n * d.pa);
  ex.partials = (double*)scr.take(sizeof(double) * (size_t)ex.partial_cap);
  if (!ex.partials) return fail(FFGB_ERR_OOM, "scratch too small for partial sums");
  int nct = 0;
  StageOpts o = stack_opts(2 * salt + 1, d.pa);
  o.expect = &ex;
  o.expect_ctas = &nct;
  FFGB_TRY(stage_rotate_rows(T, T, norb, nb, d.n * d.pa, d.n * d.pa, pv, o, st));
  FFGB_TRY(launch_state_partials(ex.partials, nct, d.n * d.pa / STACK_TILE, d.pa / STACK_TILE, d.n, slots, st));
  scr.off = mark;
  return FFGB_OK;
}

// Yacc += W(U) Z W(U)^dag psi_b for every state of the stack Y (alpha rows,
// not modified); the stage path of rotated_matvec_impl over the whole stack.
// Y1 and T are stacked scratch; T's padding columns must be zero.
static int stack_rotated_matvec(const void* Y, void* Yacc, void* Y1, void* T, const Stack& d, int norb, int na,
                                int nb, const DiagSpec& spec, const SectorPlan& pd, const SectorPlan& pu,
                                Scratch& scr, cudaStream_t st) {
  const size_t mark = scr.off;
  const long long ya = d.n * d.pb, tb = d.n * d.pa;  // row lengths of the two layouts
  const void *fa = nullptr, *fb = nullptr;
  // the final phases of pd are carried by pu (sandwich_plans)
  FFGB_TRY(stage_rotate_rows(Y, Y1, norb, na, ya, ya, pd, stack_opts(8, d.pb), st));
  FFGB_TRY(launch_transpose_stacked<float>(Y1, T, d.da, d.db, d.n, d.pb, d.pa, nullptr, st));
  FFGB_TRY(stage_rotate_rows(T, T, norb, nb, tb, tb, pd, stack_opts(9, d.pa), st));
  FFGB_TRY(diag_rows<float>(T, T, norb, nb, na, spec.transposed(), false, scr, st, nullptr, nullptr, d.n));
  scr.off = mark;
  FFGB_TRY(phase_table(&pu, norb, na, scr, st, &fa));
  FFGB_TRY(phase_table(&pu, norb, nb, scr, st, &fb));
  FFGB_TRY(stage_rotate_rows(T, T, norb, nb, tb, tb, pu, stack_opts(11, d.pa), st));
  FFGB_TRY(launch_transpose_stacked<float>(T, Y1, d.db, d.da, d.n, d.pa, d.pb, fb, st));
  FFGB_TRY(stage_rotate_rows(Y1, Y1, norb, na, ya, ya, pu, stack_opts(10, d.pb), st));
  FFGB_TRY(launch_row_axpy<float>(Y1, Yacc, d.da, ya, fa, st));
  scr.off = mark;
  return FFGB_OK;
}

// Host-side control of a batch call: cancellation and deadline checks
// between units of work (a state's circuit, a Hamiltonian term), with at most
// two units queued on the stream ahead of the GPU so that a check acts within
// about two units.
class Pacer {
 public:
  Pacer(const ffgb_control* c, cudaStream_t st) : c_(c), st_(st), t0_(std::chrono::steady_clock::now()) {}
  ~Pacer() {
    for (cudaEvent_t e : ev_)
      if (e) cudaEventDestroy(e);
  }
  // before enqueueing unit k
  int before(long long k) {
    if (!c_) return FFGB_OK;
    if (k >= 2 && ev_[k % 2]) FFGB_CUDA(cudaEventSynchronize(ev_[k % 2]));  // unit k - 2 has finished
    if (c_->cancel && *c_->cancel) return fail(FFGB_ERR_CANCELLED, "cancelled after " + std::to_string(k) + " units");
    if (c_->timeout_s > 0) {
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
      if (dt > c_->timeout_s)
        return fail(FFGB_ERR_TIMEOUT, "deadline of " + std::to_string(c_->timeout_s) + " s passed after " +
                                          std::to_string(k) + " units");
    }
    return FFGB_OK;
  }
  // after enqueueing unit k
  int after(long long k) {
    if (!c_) return FFGB_OK;
    cudaEvent_t& e = ev_[k % 2];
    if (!e) FFGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    FFGB_CUDA(cudaEventRecord(e, st_));
    return FFGB_OK;
  }

 private:
  const ffgb_control* c_;
  cudaStream_t st_;
  std::chrono::steady_clock::time_point t0_;
  cudaEvent_t ev_[2] = {nullptr, nullptr};
};

// Whether a batch runs stacked: complex64 on the stage path (every term's
// rotation a cosine-sine plan); otherwise the states run one by one.
static int stack_plans(int dtype, int norb, int na, int nb, const std::vector<Term>& terms, bool both_ways,
                       std::vector<SectorPlan>& pd, std::vector<SectorPlan>& pu, bool& stacked) {
  stacked = dtype == FFGB_C64 && nb >= 0 && !big_rows<float>(norb, na, nb);
  if (!stacked) return FFGB_OK;
  pd.resize(terms.size());
  pu.resize(both_ways ? terms.size() : 0);
  for (size_t k = 0; k < terms.size(); ++k) {
    bool stage = false;
    if (both_ways) {
      // pu[k] carries the final phases of pd[k] (sandwich_plans)
      FFGB_TRY(sandwich_plans<float>(norb, terms[k].rot, pd[k], pu[k], &stage));
    } else {
      FFGB_TRY(make_plan<float>(norb, dagger(terms[k].rot, norb), pd[k]));
      stage = staged<float>(&pd[k], nullptr);
    }
    if (!stage) stacked = false;
  }
  return FFGB_OK;
}

static Stack make_stack(long long n, int norb, int na, int nb) {
  Stack d;
  d.n = n;
  d.da = binom_h(norb, na);
  d.db = binom_h(norb, nb);
  d.pa = stack_pad(d.da);
  d.pb = stack_pad(d.db);
  return d;
}

// Energies of n contiguous states x[b] (complex64 stacked, else one by one).
static int batch_df_energy(const void* x, long long n, int dtype, int norb, int na, int nb,
                           const std::vector<Term>& terms, double constant, double* energies, Scratch& scr,
                           cudaStream_t st, Pacer& pace, long long unit0) {
  std::vector<SectorPlan> pd, pu;
  bool stacked = false;
  FFGB_TRY(stack_plans(dtype, norb, na, nb, terms, false, pd, pu, stacked));
  const long long dim = binom_h(norb, na) * binom_h(norb, nb);
  if (!stacked) {
    const size_t el = dtype == FFGB_C128 ? 16 : 8;
    for (long long b = 0; b < n; ++b) {
      FFGB_TRY(pace.before(unit0 + b));
      const size_t mark = scr.off;
      const void* xb = (const char*)x + (size_t)(b * dim) * el;
      FFGB_TRY(FFGB_DISPATCH(dtype,
                             df_expectation_impl<float>(xb, norb, na, nb, terms, nullptr, constant, energies + b,
                                                        scr, st),
                             df_expectation_impl<double>(xb, norb, na, nb, terms, nullptr, constant, energies + b,
                                                         scr, st)));
      scr.off = mark;
      FFGB_TRY(pace.after(unit0 + b));
    }
    return FFGB_OK;
  }
  const Stack d = make_stack(n, norb, na, nb);
  void* Y = scr.take(d.ybytes());
  void* Y1 = scr.take(d.ybytes());
  void* T = scr.take(d.tbytes());
  double* slots = (double*)scr.take(sizeof(double) * (size_t)(n * std::max<size_t>(terms.size(), 1)));
  if (!Y || !Y1 || !T || !slots) return fail(FFGB_ERR_OOM, "scratch too small for the stacked batch");
  FFGB_CUDA(cudaMemsetAsync(Y, 0, d.ybytes(), st));
  FFGB_CUDA(cudaMemsetAsync(T, 0, d.tbytes(), st));
  FFGB_TRY(launch_stack<float>(const_cast<void*>(x), Y, n, d.da, d.db, d.pb, 0, 0, st));
  for (size_t k = 0; k < terms.size(); ++k) {
    FFGB_TRY(pace.before(unit0 + (long long)k));
    FFGB_TRY(stack_expectation_term(Y, Y1, T, d, norb, na, nb, terms[k].spec, pd[k], slots + k * n,
                                    100u + (unsigned)k, scr, st));
    FFGB_TRY(pace.after(unit0 + (long long)k));
  }
  std::vector<double> h((size_t)n * terms.size(), 0.0);
  if (!terms.empty())
    FFGB_CUDA(cudaMemcpyAsync(h.data(), slots, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  FFGB_CUDA(cudaStreamSynchronize(st));
  for (long long b = 0; b < n; ++b) {
    double e = constant;
    for (size_t k = 0; k < terms.size(); ++k) e += h[k * n + b];
    energies[b] = e;
  }
  return FFGB_OK;
}

static size_t batch_scratch(int op, int dtype, int norb, int na, int nb, long long n) {
  const size_t el = dtype == FFGB_C128 ? 16 : 8;
  const long long da = binom_h(norb, na), db = nb >= 0 ? binom_h(norb, nb) : 1;
  const size_t S = (size_t)(da * db) * el;
  const size_t ex = extras_bytes(norb, na, nb) + 4096;
  const Stack d = make_stack(n, norb, na, std::max(nb, 0));
  // per-state path (a circuit, or states that do not stack): two states
  size_t need = 2 * S + ex;
  if (dtype == FFGB_C64 && nb >= 0) {
    const size_t partials = sizeof(double) * (size_t)stage_expect_partials(d.db, d.n * d.pa);
    // energy slots: n per term, for up to 2 norb^2 + 1 terms (a molecular
    // Hamiltonian's exact factorization has at most 2 norb^2)
    const size_t slots = (size_t)n * 8 * (2 * (size_t)norb * norb + 2);
    const size_t stack = op == 0 ? 2 * d.ybytes() + d.tbytes() + partials + slots : 3 * d.ybytes() + d.tbytes();
    need = std::max(need, stack + ex + 4096);
  }
  return need;
}

// ---------------------------------------------------------------------------
// allocation-free contraction: scratch in a fixed device array
// ---------------------------------------------------------------------------
// Every byte read from this array is written earlier in the same call, so it
// never needs clearing.  One array per device: calls that overlap in time on
// one device (other streams, other host threads) share it and race.
static __device__ __align__(256) unsigned char g_static_scratch[FFGB_STATIC_SCRATCH_BYTES];

// Occupation string of every colex rank (ascending bit patterns with nocc bits).
static __global__ void colex_strings_kernel(unsigned* __restrict__ out, int dim, int norb, int nocc) {
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t0 >= dim) return;
  int t = t0, k = nocc;
  unsigned s = 0;
  for (int p = norb - 1; p >= 0 && k > 0; --p) {
    long long c = 1;  // C(p, k)
    if (k > p) {
      c = 0;
    } else {
      for (int i = 1; i <= k; ++i) c = c * (p - k + i) / i;
    }
    if (t >= c) {
      s |= 1u << p;
      t -= (int)c;
      --k;
    }
  }
  out[t0] = s;
}

static std::mutex g_static_mu;
static void* g_static_ptr[64] = {};

// Device address of g_static_scratch on the current device, looked up once per device.
static int static_scratch(void** out) {
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FFGB_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) FFGB_CUDA(cudaGetSymbolAddress(&g_static_ptr[dev], g_static_scratch));
  *out = g_static_ptr[dev];
  return FFGB_OK;
}

static size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }

template <typename T>
static int contract_static_impl(const void* vec, void* out, int norb, int na, int nb, const DiagSpec& spec,
                                int accumulate, cudaStream_t st) {
  using C = typename CT<T>::type;
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  // the column table is built only when the beta-beta block is nonzero (run_pass)
  bool col_nonzero = false;
  for (int i = 0; i < FFGB_MAXN && !col_nonzero; ++i)
    for (int j = 0; j < FFGB_MAXN; ++j)
      if (spec.col_same[i][j] != 0.0) col_nonzero = true;
  const size_t need = round256((size_t)da * 4) + round256((size_t)db * 4) +
                      (col_nonzero ? round256((size_t)db * sizeof(C)) : 0);
  if (need > FFGB_STATIC_SCRATCH_BYTES)
    return fail(FFGB_ERR_ARG, "this shape needs " + std::to_string(need) + " bytes of scratch; the fixed scratch of "
                                  "ffgb_contract_diag_coulomb_static holds " +
                                  std::to_string((size_t)FFGB_STATIC_SCRATCH_BYTES) +
                                  " (use ffgb_contract_diag_coulomb)");
  FFGB_TRY(need_buffers({vec, out}));
  if (da <= 0 || db <= 0) return FFGB_OK;
  void* base = nullptr;
  FFGB_TRY(static_scratch(&base));
  Scratch scr(base, FFGB_STATIC_SCRATCH_BYTES);
  unsigned* sa = (unsigned*)scr.take((size_t)da * 4);
  unsigned* sb = (unsigned*)scr.take((size_t)db * 4);
  colex_strings_kernel<<<(unsigned)((da + 255) / 256), 256, 0, st>>>(sa, (int)da, norb, na);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  colex_strings_kernel<<<(unsigned)((db + 255) / 256), 256, 0, st>>>(sb, (int)db, norb, nb);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  PassArgs<T> A;
  A.norb = norb;
  A.rot_nocc = nb;
  A.row_nocc = na;
  A.n_rows = da;
  A.in = vec;
  A.out = out;
  A.out_op = accumulate ? OUT_ACCUM : OUT_STORE;
  A.diag = &spec;
  A.col_strings = sb;
  A.row_strings = sa;
  return run_pass<T>(A, scr, st);
}

// Partial-sum bytes of densities() for both sectors and both kernel forms.
static size_t density_scratch(int norb, int na, int nb) {
  size_t b = std::max(density_partial_bytes(norb, binom_h(norb, na)),
                      density_partial_bytes(norb, binom_h(norb, std::max(nb, 0))));
  for (int n : {na, nb})
    if (n >= 1) b = std::max(b, density_sub_bytes(norb, binom_h(norb, n - 1), norb - n + 1));
  return b;
}

// Densities between two states: the beta sector runs on transposed copies.
template <typename T>
static int densities(const void* x, const void* y, int norb, int na, int nb, bool pair, double* out,
                     Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  const unsigned *sa = nullptr, *sb = nullptr;
  FFGB_TRY(device_strings(norb, na, &sa));
  FFGB_TRY(device_strings(norb, nb, &sb));
  const size_t S = (size_t)(da * db) * sizeof(C);
  void* tx = scr.take(S);
  void* ty = scr.take(S);
  const size_t pbytes = density_scratch(norb, na, nb);
  void* part = scr.take(pbytes);
  // strings with one electron fewer (the transition density's sub-string form)
  const unsigned *sa1 = nullptr, *sb1 = nullptr;
  if (na >= 1) FFGB_TRY(device_strings(norb, na - 1, &sa1));
  if (nb >= 1) FFGB_TRY(device_strings(norb, nb - 1, &sb1));
  if (!tx || !ty || !part) return fail(FFGB_ERR_OOM, "scratch too small (needs two states)");
  FFGB_TRY(launch_transpose<T>(x, tx, da, db, nullptr, nullptr, st));
  FFGB_TRY(launch_transpose<T>(y, ty, da, db, nullptr, nullptr, st));
  const size_t n2 = 2 * (size_t)norb * norb;
  if (!pair) {
    std::vector<double> ga, gb;
    FFGB_TRY(rdm1_rows<T>(x, y, sa, (int)da, (int)db, norb, part, pbytes, ga, st, na, sa1,
                          na >= 1 ? (int)binom_h(norb, na - 1) : 0));
    FFGB_TRY(rdm1_rows<T>(tx, ty, sb, (int)db, (int)da, norb, part, pbytes, gb, st, nb, sb1,
                          nb >= 1 ? (int)binom_h(norb, nb - 1) : 0));
    std::memcpy(out, ga.data(), n2 * sizeof(double));
    std::memcpy(out + n2, gb.data(), n2 * sizeof(double));
  } else {
    std::vector<double> aa, ab, bb, ba;
    FFGB_TRY(pair_rows<T>(x, y, sa, sb, (int)da, (int)db, norb, part, pbytes, aa, ab, st));
    FFGB_TRY(pair_rows<T>(tx, ty, sb, sa, (int)db, (int)da, norb, part, pbytes, bb, ba, st));
    std::memcpy(out, aa.data(), n2 * sizeof(double));
    std::memcpy(out + n2, ab.data(), n2 * sizeof(double));
    std::memcpy(out + 2 * n2, bb.data(), n2 * sizeof(double));
  }
  return FFGB_OK;
}

// Both densities of one gate between x and y into device memory (no
// synchronization): out_dev = [G^alpha, G^beta] (transition 1-RDM) and, with
// `pair`, [P^aa, P^ab, P^bb] after them; norb * norb complex values each.
// One pair of transposes serves both.
template <typename T>
static int densities_dev(const void* x, const void* y, int norb, int na, int nb, bool pair, double2* out_dev,
                         Scratch& scr, cudaStream_t st) {
  using C = typename CT<T>::type;
  const long long da = binom_h(norb, na), db = binom_h(norb, nb);
  const unsigned *sa = nullptr, *sb = nullptr;
  FFGB_TRY(device_strings(norb, na, &sa));
  FFGB_TRY(device_strings(norb, nb, &sb));
  const size_t S = (size_t)(da * db) * sizeof(C);
  const size_t n2 = (size_t)norb * norb;
  void* tx = scr.take(S);
  void* ty = scr.take(S);
  const size_t pbytes = density_scratch(norb, na, nb);
  void* part = scr.take(pbytes);
  void* bbuf = scr.take(sizeof(double2) * 2 * n2);  // the beta pass's (bb, ba) sums
  const unsigned *sa1 = nullptr, *sb1 = nullptr;
  if (na >= 1) FFGB_TRY(device_strings(norb, na - 1, &sa1));
  if (nb >= 1) FFGB_TRY(device_strings(norb, nb - 1, &sb1));
  if (!tx || !ty || !part || !bbuf) return fail(FFGB_ERR_OOM, "scratch too small (needs two states)");
  FFGB_TRY(launch_transpose<T>(x, tx, da, db, nullptr, nullptr, st));
  FFGB_TRY(launch_transpose<T>(y, ty, da, db, nullptr, nullptr, st));
  FFGB_TRY(rdm1_rows_dev<T>(x, y, sa, (int)da, (int)db, norb, part, pbytes, out_dev, st, na, sa1,
                            na >= 1 ? (int)binom_h(norb, na - 1) : 0));
  FFGB_TRY(rdm1_rows_dev<T>(tx, ty, sb, (int)db, (int)da, norb, part, pbytes, out_dev + n2, st, nb, sb1,
                            nb >= 1 ? (int)binom_h(norb, nb - 1) : 0));
  if (pair) {
    FFGB_TRY(pair_rows_dev<T>(x, y, sa, sb, (int)da, (int)db, norb, part, pbytes, out_dev + 2 * n2, st));
    FFGB_TRY(pair_rows_dev<T>(tx, ty, sb, sa, (int)db, (int)da, norb, part, pbytes, (double2*)bbuf, st));
    FFGB_CUDA(cudaMemcpyAsync(out_dev + 4 * n2, bbuf, sizeof(double2) * n2, cudaMemcpyDeviceToDevice, st));
  }
  return FFGB_OK;
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int ffgb_version(void) { return 100; }

const char* ffgb_last_error(void) { return ffgb::g_err.c_str(); }

long long ffgb_launch_count(void) { return g_launches.load(); }

long long ffgb_device_alloc_count(void) { return g_allocs.load(); }

int ffgb_givens_decomposition(const double* mat, int n, double tol, double* rot_cs, int* rot_ij,
                              int* n_rot, double* diag) {
  g_err.clear();
  if (!mat || n < 0) return fail(FFGB_ERR_ARG, "mat must be a square matrix");
  std::vector<RefGivens> rots;
  std::vector<cd> d;
  reference_givens_decomposition(n, load_mat(mat, n).data(), tol, rots, d);
  for (size_t k = 0; k < rots.size(); ++k) {
    rot_cs[3 * k] = rots[k].c;
    rot_cs[3 * k + 1] = rots[k].s.real();
    rot_cs[3 * k + 2] = rots[k].s.imag();
    rot_ij[2 * k] = rots[k].i;
    rot_ij[2 * k + 1] = rots[k].j;
  }
  *n_rot = (int)rots.size();
  for (int i = 0; i < n; ++i) {
    diag[2 * i] = d[i].real();
    diag[2 * i + 1] = d[i].imag();
  }
  return FFGB_OK;
}

int ffgb_eigh(const double* mat, int n, double* eigvals, double* vecs) {
  g_err.clear();
  if (!mat || n < 0) return fail(FFGB_ERR_ARG, "invalid matrix");
  std::vector<double> w;
  std::vector<cd> v;
  hermitian_eigh(n, load_mat(mat, n).data(), w, v);
  for (int i = 0; i < n; ++i) eigvals[i] = w[i];
  for (size_t i = 0; i < v.size(); ++i) {
    vecs[2 * i] = v[i].real();
    vecs[2 * i + 1] = v[i].imag();
  }
  return FFGB_OK;
}

int ffgb_debug_plan(const double* mat, int norb, int use_windows, double* out, int cap, int* len) {
  g_err.clear();
  SectorPlan p;
  if (!plan_sector(norb, load_mat(mat, norb).data(), use_windows != 0, p))
    return fail(FFGB_ERR_NUMERIC, "plan failed");
  std::vector<double> o;
  o.push_back(p.kind);
  o.push_back(p.h);
  o.push_back(p.max_err);
  auto put_g = [&](const std::vector<Givens>& v) {
    o.push_back((double)v.size());
    for (auto& g : v) {
      o.push_back(g.c);
      o.push_back(g.s.real());
      o.push_back(g.s.imag());
    }
  };
  put_g(p.tri);
  put_g(p.b1);
  put_g(p.b2);
  put_g(p.a1);
  put_g(p.a2);
  o.push_back((double)p.cs.size());
  for (auto& c : p.cs) {
    o.push_back(c.i);
    o.push_back(c.j);
    for (cd z : {c.g00, c.g01, c.g10, c.g11}) {
      o.push_back(z.real());
      o.push_back(z.imag());
    }
  }
  // the five-stage form's phases, then the stage sequence with its phases
  const std::vector<cd>& d5 = p.kind == PLAN_CSD ? p.csd_diag : p.diag;
  o.push_back((double)d5.size());
  for (cd z : d5) {
    o.push_back(z.real());
    o.push_back(z.imag());
  }
  o.push_back((double)p.ops.size());
  for (const StageOp& op : p.ops) {
    o.push_back(op.type);
    o.push_back(op.lo);
    o.push_back(op.b);
    put_g(op.net);
    o.push_back((double)op.pairs.size());
    for (auto& c : op.pairs) {
      o.push_back(c.i);
      o.push_back(c.j);
      for (cd z : {c.g00, c.g01, c.g10, c.g11}) {
        o.push_back(z.real());
        o.push_back(z.imag());
      }
    }
  }
  o.push_back((double)p.diag.size());
  for (cd z : p.diag) {
    o.push_back(z.real());
    o.push_back(z.imag());
  }
  if ((int)o.size() > cap) return fail(FFGB_ERR_ARG, "output buffer too small");
  std::memcpy(out, o.data(), o.size() * sizeof(double));
  *len = (int)o.size();
  return FFGB_OK;
}

int ffgb_debug_stage(void* vec, int dtype, int norb, int na, int nb, const double* mat, int stage,
                     void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  if (dtype != FFGB_C64 || nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "stage kernels run on spinful complex64 states");
  if (!mat) return fail(FFGB_ERR_ARG, "mat must not be NULL");
  SectorPlan p;
  FFGB_TRY(make_plan<float>(norb, load_mat(mat, norb), p));
  if (p.kind != PLAN_CSD) return fail(FFGB_ERR_UNSUPPORTED, "no cosine-sine plan for this norb");
  StageOpts o;
  o.mode = STAGE_MODE;
  o.only_stage = stage;
  const long long db = binom_h(norb, nb);
  return stage_rotate_rows(vec, vec, norb, na, db, db, p, o, (cudaStream_t)stream);
}

size_t ffgb_scratch_bytes(int op, int dtype, int norb, int na, int nb) {
  const size_t el = dtype == FFGB_C128 ? 16 : 8;
  const long long da = binom_h(norb, na), db = nb >= 0 ? binom_h(norb, nb) : 1;
  const size_t S = (size_t)da * db * el;
  const size_t ex = extras_bytes(norb, na, nb) + 4096;
  if (op == 1 || op == 2) return 2 * S + ex;
  if (op == 3) return 2 * S + density_scratch(norb, na, std::max(nb, 0)) + 32 * (size_t)norb * norb + 256 + ex;
  return S + ex;
}


int ffgb_apply_givens_rotation(void* vec, int dtype, int norb, int na, int nb, int spin, double c,
                               double s_re, double s_im, int i, int j, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  if (spin != 0 && spin != 1) return fail(FFGB_ERR_ARG, "spin must be 0 (alpha) or 1 (beta)");
  if (nb < 0 && spin != 0) return fail(FFGB_ERR_ARG, "spinless systems have one sector");
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, givens_impl<float>(vec, norb, na, nb, spin, c, s_re, s_im, i, j, st),
                       givens_impl<double>(vec, norb, na, nb, spin, c, s_re, s_im, i, j, st));
}

int ffgb_apply_phase_shift(void* vec, int dtype, int norb, int na, int nb, int spin, double pr,
                           double pi, int orb, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  if (orb < 0 || orb >= norb) return fail(FFGB_ERR_ARG, "orbital index out of range");
  cudaStream_t st = (cudaStream_t)stream;
  const int nocc = (spin == 0 || nb < 0) ? na : nb;
  const unsigned* strs = nullptr;
  FFGB_TRY(device_strings(norb, nocc, &strs));
  const long long da = binom_h(norb, na), db = nb < 0 ? 1 : binom_h(norb, nb);
  const int sp = nb < 0 ? 0 : spin;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((da * db + 255) / 256, 8192));
  if (dtype == FFGB_C64)
    phase_shift_kernel<float><<<blocks, 256, 0, st>>>((float2*)vec, strs, da, db, sp, orb, (float)pr, (float)pi);
  else
    phase_shift_kernel<double><<<blocks, 256, 0, st>>>((double2*)vec, strs, da, db, sp, orb, pr, pi);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

int ffgb_apply_excitation(const void* vec, void* out, int dtype, int norb, int na, int nb, int spin, int p, int q,
                          void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  if (!vec || !out || vec == out) return fail(FFGB_ERR_ARG, "vec and out must be distinct device buffers");
  if (p < 0 || q < 0 || p >= norb || q >= norb) return fail(FFGB_ERR_ARG, "orbital index out of range");
  if (spin != 0 && spin != 1) return fail(FFGB_ERR_ARG, "spin must be 0 (alpha) or 1 (beta)");
  if (nb < 0 && spin != 0) return fail(FFGB_ERR_ARG, "spinless systems have one sector");
  cudaStream_t st = (cudaStream_t)stream;
  const int sp = nb < 0 ? 0 : spin;
  const int nocc = sp == 0 ? na : nb;
  const long long da = binom_h(norb, na), db = nb < 0 ? 1 : binom_h(norb, nb);
  const size_t el = dtype == FFGB_C64 ? sizeof(float2) : sizeof(double2);
  FFGB_CUDA(cudaMemsetAsync(out, 0, (size_t)(da * db) * el, st));
  if (nocc == 0 || da * db == 0) return FFGB_OK;
  const unsigned* strs = nullptr;
  FFGB_TRY(device_strings(norb, nocc, &strs));
  const int blocks = (int)std::max<long long>(1, std::min<long long>((da * db + 255) / 256, 8192));
  if (dtype == FFGB_C64)
    excitation_kernel<float><<<blocks, 256, 0, st>>>((const float2*)vec, (float2*)out, strs, da, db, sp, p, q);
  else
    excitation_kernel<double><<<blocks, 256, 0, st>>>((const double2*)vec, (double2*)out, strs, da, db, sp, p, q);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

int ffgb_apply_orbital_rotation(void* vec, int dtype, int norb, int na, int nb, const double* ma,
                                const double* mb, void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, orbital_rotation_impl<float>(vec, norb, na, nb, ma, mb, scr, st),
                       orbital_rotation_impl<double>(vec, norb, na, nb, ma, mb, scr, st));
}

int ffgb_apply_diag_coulomb_evolution(void* vec, int dtype, int norb, int na, int nb,
                                      const double* aa, const double* ab, const double* bb,
                                      double time, int zrep, const double* rot_a,
                                      const double* rot_b, void* scratch, size_t scratch_bytes,
                                      void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  if (nb < 0 && zrep) return fail(FFGB_ERR_UNSUPPORTED, "Z representation needs a spinful system");
  DiagSpec spec = diag_coulomb_spec(norb, aa, nb < 0 ? nullptr : ab, nb < 0 ? nullptr : bb, zrep,
                                    -time, DIAG_PHASE);
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype,
                       diag_evolution_impl<float>(vec, norb, na, nb, spec, rot_a, rot_b, scr, st),
                       diag_evolution_impl<double>(vec, norb, na, nb, spec, rot_a, rot_b, scr, st));
}

int ffgb_apply_num_op_sum_evolution(void* vec, int dtype, int norb, int na, int nb,
                                    const double* ca, const double* cb, double time,
                                    const double* rot_a, const double* rot_b, void* scratch,
                                    size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  DiagSpec spec = one_body_spec(norb, ca, nb < 0 ? nullptr : cb, -time, DIAG_PHASE);
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype,
                       diag_evolution_impl<float>(vec, norb, na, nb, spec, rot_a, rot_b, scr, st),
                       diag_evolution_impl<double>(vec, norb, na, nb, spec, rot_a, rot_b, scr, st));
}

int ffgb_ucj_spin_balanced_apply(void* vec, int dtype, int norb, int na, int nb, int n_reps,
                                 const double* dcm, const double* rots, const double* final_rot,
                                 void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "spin-balanced UCJ needs a spinful system");
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t el = dtype == FFGB_C128 ? 16 : 8;
  void* tmp = scr.take((size_t)binom_h(norb, na) * binom_h(norb, nb) * el);
  if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
  std::vector<cd> current = eye(norb);
  for (int k = 0; k < n_reps; ++k) {
    std::vector<cd> U = load_mat(rots + (size_t)k * norb * norb * 2, norb);
    std::vector<cd> V = matmul(dagger(U, norb), current, norb);
    const double* J = dcm + (size_t)k * 2 * norb * norb;
    DiagSpec spec = diag_coulomb_spec(norb, J, J + norb * norb, J, 0, 1.0, DIAG_PHASE);
    SectorPlan p;
    int s = dtype == FFGB_C64 ? make_plan<float>(norb, V, p) : make_plan<double>(norb, V, p);
    if (s) return s;
    s = dtype == FFGB_C64 ? ucj_layer<float>(vec, tmp, norb, na, nb, p, &spec, 20u + (unsigned)k, scr, st)
                          : ucj_layer<double>(vec, tmp, norb, na, nb, p, &spec, 0, scr, st);
    if (s) return s;
    current = U;
  }
  std::vector<cd> V = final_rot ? matmul(load_mat(final_rot, norb), current, norb) : current;
  SectorPlan p;
  int s = dtype == FFGB_C64 ? make_plan<float>(norb, V, p) : make_plan<double>(norb, V, p);
  if (s) return s;
  return dtype == FFGB_C64 ? ucj_layer<float>(vec, tmp, norb, na, nb, p, nullptr, 19u, scr, st)
                           : ucj_layer<double>(vec, tmp, norb, na, nb, p, nullptr, 0, scr, st);
}

int ffgb_contract_diag_coulomb(const void* vec, void* out, int dtype, int norb, int na, int nb,
                               const double* aa, const double* ab, const double* bb, int zrep,
                               int accumulate, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "contraction needs a spinful system");
  DiagSpec spec = diag_coulomb_spec(norb, aa, ab, bb, zrep, 1.0, DIAG_COEF);
  char buf[1];
  Scratch scr(nullptr, 0);
  (void)buf;
  cudaStream_t st = (cudaStream_t)stream;
  // the column table needs scratch; use a small internal allocation per call
  const size_t need = (size_t)binom_h(norb, nb) * 16 + 8192;
  void* tmp = nullptr;
  FFGB_CUDA(cudaMallocAsync(&tmp, need, st));
  count_alloc();
  Scratch s2(tmp, need);
  int s = FFGB_DISPATCH(dtype, rotated_matvec_impl<float>(vec, out, norb, na, nb, spec, nullptr, accumulate, s2, st),
                        rotated_matvec_impl<double>(vec, out, norb, na, nb, spec, nullptr, accumulate, s2, st));
  cudaFreeAsync(tmp, st);
  return s;
}

int ffgb_contract_diag_coulomb_static(const void* vec, void* out, int dtype, int norb, int na, int nb,
                                      const double* aa, const double* ab, const double* bb, int zrep,
                                      int accumulate, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "contraction needs a spinful system");
  DiagSpec spec = diag_coulomb_spec(norb, aa, ab, bb, zrep, 1.0, DIAG_COEF);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, contract_static_impl<float>(vec, out, norb, na, nb, spec, accumulate, st),
                       contract_static_impl<double>(vec, out, norb, na, nb, spec, accumulate, st));
}

int ffgb_contract_num_op_sum(const void* vec, void* out, int dtype, int norb, int na, int nb,
                             const double* coeffs, int accumulate, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "contraction needs a spinful system");
  DiagSpec spec = one_body_spec(norb, coeffs, coeffs, 1.0, DIAG_COEF);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t need = (size_t)binom_h(norb, nb) * 16 + 8192;
  void* tmp = nullptr;
  FFGB_CUDA(cudaMallocAsync(&tmp, need, st));
  count_alloc();
  Scratch s2(tmp, need);
  int s = FFGB_DISPATCH(dtype, rotated_matvec_impl<float>(vec, out, norb, na, nb, spec, nullptr, accumulate, s2, st),
                        rotated_matvec_impl<double>(vec, out, norb, na, nb, spec, nullptr, accumulate, s2, st));
  cudaFreeAsync(tmp, st);
  return s;
}

int ffgb_rotated_diag_matvec(const void* vec, void* out, int dtype, int norb, int na, int nb,
                             const double* one_body, const double* mat, int zrep, const double* rot,
                             int accumulate, void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "linear operator needs a spinful system");
  DiagSpec spec;
  spec.mode = DIAG_COEF;
  if (mat) spec = diag_coulomb_spec(norb, mat, mat, mat, zrep, 1.0, DIAG_COEF);
  if (one_body) add_spec(spec, one_body_spec(norb, one_body, one_body, 1.0, DIAG_COEF));
  std::vector<cd> R;
  if (rot) R = load_mat(rot, norb);
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype,
                       rotated_matvec_impl<float>(vec, out, norb, na, nb, spec, rot ? &R : nullptr, accumulate, scr, st),
                       rotated_matvec_impl<double>(vec, out, norb, na, nb, spec, rot ? &R : nullptr, accumulate, scr, st));
}

int ffgb_df_matvec(const void* vec, void* out, int dtype, int norb, int na, int nb,
                   const double* one_body, int n_terms, const double* dcm, const double* rots,
                   double constant, int zrep, void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "linear operator needs a spinful system");
  if (vec == out) return fail(FFGB_ERR_ARG, "out must not alias vec");
  std::vector<Term> terms;
  df_terms(norb, one_body, n_terms, dcm, rots, zrep, terms);
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = binom_h(norb, na) * binom_h(norb, nb);
  const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
  if (dtype == FFGB_C64)
    scale_copy_kernel<float><<<blocks, 256, 0, st>>>((const float2*)vec, (float2*)out, n, (float)constant, 0.f);
  else
    scale_copy_kernel<double><<<blocks, 256, 0, st>>>((const double2*)vec, (double2*)out, n, constant, 0.0);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  for (const Term& t : terms) {
    const size_t mark = scr.off;
    int s = FFGB_DISPATCH(dtype,
                          rotated_matvec_impl<float>(vec, out, norb, na, nb, t.spec, &t.rot, 1, scr, st),
                          rotated_matvec_impl<double>(vec, out, norb, na, nb, t.spec, &t.rot, 1, scr, st));
    if (s) return s;
    scr.off = mark;
  }
  return FFGB_OK;
}

int ffgb_df_expectation(const void* vec, int dtype, int norb, int na, int nb, const double* one_body,
                        int n_terms, const double* dcm, const double* rots, double constant,
                        int zrep, const double* pre_rotation, double* energy_out, void* scratch,
                        size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, energy_out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "expectation needs a spinful system");
  std::vector<Term> terms;
  df_terms(norb, one_body, n_terms, dcm, rots, zrep, terms);
  std::vector<cd> pre;
  if (pre_rotation) pre = load_mat(pre_rotation, norb);
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype,
                       df_expectation_impl<float>(vec, norb, na, nb, terms, pre_rotation ? &pre : nullptr, constant, energy_out, scr, st),
                       df_expectation_impl<double>(vec, norb, na, nb, terms, pre_rotation ? &pre : nullptr, constant, energy_out, scr, st));
}

int ffgb_lucj_energy(const void* vec_in, void* work, int dtype, int norb, int na, int nb, int n_reps,
                     const double* ucj_dcm, const double* ucj_rots, const double* ucj_final,
                     const double* one_body, int n_terms, const double* dcm, const double* rots,
                     double constant, double* energy_out, void* scratch, size_t scratch_bytes,
                     void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({work, energy_out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "LUCJ energy needs a spinful system");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t el = dtype == FFGB_C128 ? 16 : 8;
  const long long n = binom_h(norb, na) * binom_h(norb, nb);
  // from the Hartree-Fock state the first layer is a Slater determinant (below)
  const bool slater_start = !vec_in && n_reps >= 1;
  if (vec_in) {
    FFGB_CUDA(cudaMemcpyAsync(work, vec_in, (size_t)n * el, cudaMemcpyDeviceToDevice, st));
  } else if (!slater_start) {
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    if (dtype == FFGB_C64)
      one_hot_kernel<float><<<blocks, 256, 0, st>>>((float2*)work, n);
    else
      one_hot_kernel<double><<<blocks, 256, 0, st>>>((double2*)work, n);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
  }
  Scratch scr(scratch, scratch_bytes);
  void* tmp = scr.take((size_t)n * el);
  if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
  std::vector<cd> current;
  FFGB_TRY(ucj_layers(work, tmp, dtype, norb, na, nb, n_reps, ucj_dcm, ucj_rots, slater_start, scr, st, current));
  std::vector<cd> final_basis = ucj_final ? matmul(load_mat(ucj_final, norb), current, norb) : current;
  std::vector<Term> terms;
  df_terms(norb, one_body, n_terms, dcm, rots, 0, terms);
  scr.off = 0;
  return FFGB_DISPATCH(dtype,
                       df_expectation_impl<float>(work, norb, na, nb, terms, &final_basis, constant, energy_out, scr, st),
                       df_expectation_impl<double>(work, norb, na, nb, terms, &final_basis, constant, energy_out, scr, st));
}

size_t ffgb_batch_scratch_bytes(int op, int dtype, int norb, int na, int nb, long long n_states) {
  if (n_states <= 0 || norb < 0 || norb > FFGB_MAXN) return 0;
  return batch_scratch(op, dtype, norb, na, nb, n_states);
}

int ffgb_batch_lucj_energy(void* work, long long n_states, int dtype, int norb, int na, int nb, int n_reps,
                           const double* ucj_dcm, const double* ucj_rots, const double* ucj_final,
                           const double* one_body, int n_terms, const double* dcm, const double* rots,
                           double constant, double* energies_out, void* scratch, size_t scratch_bytes,
                           const ffgb_control* control, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({work, energies_out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "LUCJ energy needs a spinful system");
  if (n_states <= 0) return fail(FFGB_ERR_ARG, "n_states must be positive");
  if (n_reps < 1) return fail(FFGB_ERR_ARG, "a batch needs n_reps >= 1");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t el = dtype == FFGB_C128 ? 16 : 8;
  const long long dim = binom_h(norb, na) * binom_h(norb, nb);
  Scratch scr(scratch, scratch_bytes);
  Pacer pace(control, st);
  {
    // each state's circuit, with its last rotation applied (it cannot merge
    // into the shared Hamiltonian terms)
    const size_t mark = scr.off;
    void* tmp = scr.take((size_t)dim * el);
    if (!tmp) return fail(FFGB_ERR_OOM, "scratch too small (needs one state)");
    const size_t per_dcm = (size_t)n_reps * 2 * norb * norb, per_rot = (size_t)n_reps * norb * norb * 2;
    for (long long b = 0; b < n_states; ++b) {
      FFGB_TRY(pace.before(b));
      void* xb = (char*)work + (size_t)(b * dim) * el;
      std::vector<cd> basis;
      FFGB_TRY(ucj_layers(xb, tmp, dtype, norb, na, nb, n_reps, ucj_dcm + b * per_dcm, ucj_rots + b * per_rot, true,
                          scr, st, basis));
      if (ucj_final) basis = matmul(load_mat(ucj_final + (size_t)b * norb * norb * 2, norb), basis, norb);
      std::vector<double> m(2 * (size_t)norb * norb);
      for (size_t i = 0; i < basis.size(); ++i) {
        m[2 * i] = basis[i].real();
        m[2 * i + 1] = basis[i].imag();
      }
      const size_t mark2 = scr.off;
      FFGB_TRY(FFGB_DISPATCH(dtype,
                             orbital_rotation_impl<float>(xb, norb, na, nb, m.data(), m.data(), scr, st),
                             orbital_rotation_impl<double>(xb, norb, na, nb, m.data(), m.data(), scr, st)));
      scr.off = mark2;
      FFGB_TRY(pace.after(b));
    }
    scr.off = mark;
  }
  std::vector<Term> terms;
  df_terms(norb, one_body, n_terms, dcm, rots, 0, terms);
  return batch_df_energy(work, n_states, dtype, norb, na, nb, terms, constant, energies_out, scr, st, pace,
                         n_states);
}

int ffgb_batch_df_matvec(const void* vec, void* out, long long n_states, int dtype, int norb, int na, int nb,
                         const double* one_body, int n_terms, const double* dcm, const double* rots, double constant,
                         int zrep, void* scratch, size_t scratch_bytes, const ffgb_control* control, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({vec, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "linear operator needs a spinful system");
  if (n_states <= 0) return fail(FFGB_ERR_ARG, "n_states must be positive");
  if (vec == out) return fail(FFGB_ERR_ARG, "out must not alias vec");
  std::vector<Term> terms;
  df_terms(norb, one_body, n_terms, dcm, rots, zrep, terms);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<SectorPlan> pd, pu;
  bool stacked = false;
  FFGB_TRY(stack_plans(dtype, norb, na, nb, terms, true, pd, pu, stacked));
  const long long dim = binom_h(norb, na) * binom_h(norb, nb);
  Pacer pace(control, st);
  if (!stacked) {
    const size_t el = dtype == FFGB_C128 ? 16 : 8;
    for (long long b = 0; b < n_states; ++b) {
      FFGB_TRY(pace.before(b));
      FFGB_TRY(ffgb_df_matvec((const char*)vec + (size_t)(b * dim) * el, (char*)out + (size_t)(b * dim) * el,
                              dtype, norb, na, nb, one_body, n_terms, dcm, rots, constant, zrep, scratch,
                              scratch_bytes, stream));
      FFGB_TRY(pace.after(b));
    }
    return FFGB_OK;
  }
  Scratch scr(scratch, scratch_bytes);
  const Stack d = make_stack(n_states, norb, na, nb);
  void* Y = scr.take(d.ybytes());
  void* Yacc = scr.take(d.ybytes());
  void* Y1 = scr.take(d.ybytes());
  void* T = scr.take(d.tbytes());
  if (!Y || !Yacc || !Y1 || !T) return fail(FFGB_ERR_OOM, "scratch too small for the stacked batch");
  FFGB_CUDA(cudaMemsetAsync(Y, 0, d.ybytes(), st));
  FFGB_CUDA(cudaMemsetAsync(Yacc, 0, d.ybytes(), st));
  FFGB_CUDA(cudaMemsetAsync(T, 0, d.tbytes(), st));
  FFGB_TRY(launch_stack<float>(const_cast<void*>(vec), Y, n_states, d.da, d.db, d.pb, 0, 0, st));
  const long long n = n_states * dim;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
  scale_copy_kernel<float><<<blocks, 256, 0, st>>>((const float2*)vec, (float2*)out, n, (float)constant, 0.f);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  for (size_t k = 0; k < terms.size(); ++k) {
    FFGB_TRY(pace.before((long long)k));
    FFGB_TRY(stack_rotated_matvec(Y, Yacc, Y1, T, d, norb, na, nb, terms[k].spec, pd[k], pu[k], scr, st));
    FFGB_TRY(pace.after((long long)k));
  }
  return launch_stack<float>(out, Yacc, n_states, d.da, d.db, d.pb, 1, 1, st);
}

int ffgb_transition_rdm1(const void* x, const void* y, int dtype, int norb, int na, int nb, double* out,
                         void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({x, y, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "densities need a spinful system");
  if (!out) return fail(FFGB_ERR_ARG, "out must not be NULL");
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, densities<float>(x, y, norb, na, nb, false, out, scr, st),
                       densities<double>(x, y, norb, na, nb, false, out, scr, st));
}

int ffgb_pair_density(const void* x, const void* y, int dtype, int norb, int na, int nb, double* out,
                      void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({x, y, out}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "densities need a spinful system");
  if (!out) return fail(FFGB_ERR_ARG, "out must not be NULL");
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, densities<float>(x, y, norb, na, nb, true, out, scr, st),
                       densities<double>(x, y, norb, na, nb, true, out, scr, st));
}

int ffgb_gate_densities(const void* x, const void* y, int dtype, int norb, int na, int nb, int pair, void* out_dev,
                        void* scratch, size_t scratch_bytes, void* stream) {
  g_err.clear();
  FFGB_TRY(check_shape(dtype, norb, na, nb));
  FFGB_TRY(need_buffers({x, y, out_dev}));
  if (nb < 0) return fail(FFGB_ERR_UNSUPPORTED, "densities need a spinful system");
  Scratch scr(scratch, scratch_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  return FFGB_DISPATCH(dtype, densities_dev<float>(x, y, norb, na, nb, pair != 0, (double2*)out_dev, scr, st),
                       densities_dev<double>(x, y, norb, na, nb, pair != 0, (double2*)out_dev, scr, st));
}

int ffgb_vdot(const void* x, const void* y, int dtype, long long n, double* out, void* stream) {
  g_err.clear();
  FFGB_TRY(need_buffers({x, y, out}));
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024));
  if (dtype != FFGB_C64 && dtype != FFGB_C128)
    return fail(FFGB_ERR_DTYPE, "dtype must be complex64 or complex128");
  double* part = nullptr;
  FFGB_CUDA(cudaMallocAsync(&part, sizeof(double) * (2 * blocks + 2), st));
  count_alloc();
  if (dtype == FFGB_C64)
    vdot_kernel<float><<<blocks, 256, 0, st>>>((const float2*)x, (const float2*)y, n, part);
  else
    vdot_kernel<double><<<blocks, 256, 0, st>>>((const double2*)x, (const double2*)y, n, part);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  std::vector<double> h(2 * blocks);
  FFGB_CUDA(cudaMemcpyAsync(h.data(), part, sizeof(double) * 2 * blocks, cudaMemcpyDeviceToHost, st));
  FFGB_CUDA(cudaStreamSynchronize(st));
  cudaFreeAsync(part, st);
  double a = 0, b = 0;
  for (int i = 0; i < blocks; ++i) {
    a += h[2 * i];
    b += h[2 * i + 1];
  }
  out[0] = a;
  out[1] = b;
  return FFGB_OK;
}

int ffgb_hartree_fock(void* vec, int dtype, long long n, void* stream) {
  g_err.clear();
  if (dtype != FFGB_C64 && dtype != FFGB_C128)
    return fail(FFGB_ERR_DTYPE, "dtype must be complex64 or complex128");
  FFGB_TRY(need_buffers({vec}));
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096));
  if (dtype == FFGB_C64)
    one_hot_kernel<float><<<blocks, 256, 0, st>>>((float2*)vec, n);
  else
    one_hot_kernel<double><<<blocks, 256, 0, st>>>((double2*)vec, n);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

}  // extern "C"
