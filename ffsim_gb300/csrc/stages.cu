// Host side of the stage-major complex64 path (see stages.cuh).
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.h"
#include "plan.h"
#include "stages.cuh"

namespace ffgb {

namespace {

long long C(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

unsigned unrank(long long t, int nbits, int k) {
  unsigned s = 0;
  for (int p = nbits - 1; p >= 0 && k > 0; --p) {
    const long long c = C(p, k);
    if (t >= c) {
      s |= 1u << p;
      t -= c;
      --k;
    }
  }
  return s;
}

long long rank(unsigned s) {
  long long r = 0;
  int t = 0;
  for (int p = 0; s; ++p, s >>= 1)
    if (s & 1u) r += C(p, ++t);
  return r;
}

long long rank_shifted(unsigned s, int base, int m0) {
  long long r = 0;
  int t = m0;
  for (int p = 0; s; ++p, s >>= 1)
    if (s & 1u) r += C(base + p, ++t);
  return r;
}

// Half-sector rank tables of a sector (norb, nocc) split at h: for every
// subset s2 of the q = norb - h high orbitals with m bits (colex index g),
// rt[moff[m] + g] = rank contribution of s2 above a low part of nocc - m electrons.
struct HalfTables {
  int h, q;
  std::vector<int> moff, rt;
};

HalfTables half_tables(int norb, int nocc, int h) {
  HalfTables t;
  t.h = h;
  t.q = norb - h;
  t.moff.assign(t.q + 2, 0);
  for (int m = 0; m <= t.q; ++m) t.moff[m + 1] = t.moff[m] + (int)C(t.q, m);
  t.rt.assign(t.moff[t.q + 1], 0);
  for (int m = 0; m <= t.q; ++m)
    for (long long g = 0; g < C(t.q, m); ++g) {
      const int m0 = nocc - m;
      t.rt[t.moff[m] + g] = (m0 >= 0 && m0 <= h) ? (int)rank_shifted(unrank(g, t.q, m), h, m0) : 0;
    }
  return t;
}

struct CsTables {
  std::vector<int*> pairs;  // device, per site
  std::vector<int> counts;
};

std::mutex g_cs_mu;
std::map<std::tuple<int, int, int, int>, CsTables> g_cs;

// Pair tables of the cross-half rotations (i, h + i) of a sector: every string
// with i occupied and h + i empty, its partner, and the parity of the occupied
// orbitals strictly between i and h + i.
int cs_tables(int norb, int nocc, int h, const CsTables** out) {
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cs_mu);
  auto key = std::make_tuple(dev, norb, nocc, h);
  auto it = g_cs.find(key);
  if (it != g_cs.end()) {
    *out = &it->second;
    return FFGB_OK;
  }
  CsTables t;
  const long long dim = C(norb, nocc);
  for (int i = 0; i < h; ++i) {
    const int j = h + i;
    const unsigned between = ((1u << j) - 1u) & ~((1u << (i + 1)) - 1u);
    std::vector<int> host;
    for (long long a = 0; a < dim; ++a) {
      const unsigned s = unrank(a, norb, nocc);
      if (!((s >> i) & 1u) || ((s >> j) & 1u)) continue;
      const unsigned y = s ^ (1u << i) ^ (1u << j);
      const int sign = __builtin_popcount(s & between) & 1;
      host.push_back((int)a | (sign ? (int)0x80000000u : 0));
      host.push_back((int)rank(y));
    }
    int* d = nullptr;
    const size_t bytes = std::max<size_t>(host.size(), 2) * sizeof(int);
    FFGB_CUDA(cudaMalloc(&d, bytes));
    if (!host.empty()) FFGB_CUDA(cudaMemcpy(d, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice));
    t.pairs.push_back(d);
    t.counts.push_back((int)(host.size() / 2));
  }
  g_cs[key] = t;
  *out = &g_cs[key];
  return FFGB_OK;
}

template <int B>
int launch_win(const WinStageParams& P, int grid, cudaStream_t st) {
  win_stage_kernel<B><<<grid, STAGE_THREADS, 0, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

int launch_win_b(int b, const WinStageParams& P, int grid, cudaStream_t st) {
  switch (b) {
    case 4: return launch_win<4>(P, grid, st);
    case 5: return launch_win<5>(P, grid, st);
    case 6: return launch_win<6>(P, grid, st);
    case 7: return launch_win<7>(P, grid, st);
    case 8: return launch_win<8>(P, grid, st);
    default: return fail(FFGB_ERR_UNSUPPORTED, "window size outside [4, 8]");
  }
}

float lo32(double x) { return (float)(x - (double)(float)x); }

// One window stage.  low: window [0, h) with groups = high-half patterns;
// otherwise window [h, norb) with groups = low-half patterns.
int window_stage(const float2* in, float2* out, long long ld, long long ncols, int norb, int nocc,
                 const HalfTables& T, bool low, const std::vector<Givens>& net, bool comp,
                 const float2* ph_in, const float2* ph_out, cudaStream_t st) {
  const int h = T.h, q = T.q;
  const int b = low ? h : q;
  auto P = std::make_unique<WinStageParams>();
  std::memset(P.get(), 0, sizeof(WinStageParams));
  P->in = in;
  P->out = out;
  P->ld = ld;
  P->ncols = ncols;
  P->low = low ? 1 : 0;
  P->comp = comp ? 1 : 0;
  P->ph_in = ph_in;
  P->ph_out = ph_out;
  for (int j = 0; j < 72; ++j) P->ident[j] = j;
  for (size_t g = 0; g < net.size(); ++g) {
    P->gp[3 * g] = (float)net[g].c;
    P->gp[3 * g + 1] = (float)net[g].s.real();
    P->gp[3 * g + 2] = (float)net[g].s.imag();
    P->gl[3 * g] = lo32(net[g].c);
    P->gl[3 * g + 1] = lo32(net[g].s.real());
    P->gl[3 * g + 2] = lo32(net[g].s.imag());
  }
  P->tiles = (int)((ncols + STAGE_THREADS - 1) / STAGE_THREADS);
  // classes: k electrons inside the window
  const int kbeg = low ? std::max(0, nocc - q) : std::max(0, nocc - h);
  const int kend = low ? std::min(h, nocc) : std::min(q, nocc);
  std::vector<int> ks;
  for (int k = kbeg; k <= kend; ++k) ks.push_back(k);
  std::stable_sort(ks.begin(), ks.end(), [&](int a, int c) { return C(b, a) > C(b, c); });
  int cta = 0, toff = 0;
  P->n_classes = (int)ks.size();
  for (size_t ci = 0; ci < ks.size(); ++ci) {
    const int k = ks[ci];
    P->cls_k[ci] = k;
    P->cls_cta0[ci] = cta;
    P->cls_off[ci] = toff;
    long long groups;
    if (low) {  // groups: high-half patterns with nocc - k electrons, base row = rt
      const int m = nocc - k;
      groups = C(q, m);
      for (long long g = 0; g < groups; ++g) P->tab[toff + g] = T.rt[T.moff[m] + g];
      toff += (int)groups;
    } else {  // groups: low-half patterns (row = colex rank), members at rt offsets
      groups = C(h, nocc - k);
      for (long long j = 0; j < C(q, k); ++j) P->tab[toff + j] = T.rt[T.moff[k] + j];
      toff += (int)C(q, k);
    }
    if (toff > 256) return fail(FFGB_ERR_UNSUPPORTED, "window table overflow");
    cta += (int)(groups * P->tiles);
  }
  P->cls_cta0[ks.size()] = cta;
  if (cta == 0) return FFGB_OK;
  return launch_win_b(b, *P, cta, st);
}

int cs_stage(float2* x, long long ld, long long ncols, int norb, int nocc, int h,
             const std::vector<Pair2>& cs, bool comp, cudaStream_t st) {
  const CsTables* T = nullptr;
  FFGB_TRY(cs_tables(norb, nocc, h, &T));
  for (size_t i = 0; i < cs.size(); ++i) {
    const int n = T->counts[i];
    if (n == 0) continue;
    CsSiteParams P;
    std::memset(&P, 0, sizeof(P));
    P.x = x;
    P.ld = ld;
    P.ncols = ncols;
    P.pairs = T->pairs[i];
    P.n_pairs = n;
    P.ppc = 8;
    P.tiles = (int)((ncols + STAGE_THREADS - 1) / STAGE_THREADS);
    P.comp = comp ? 1 : 0;
    const double v[8] = {cs[i].g00.real(), cs[i].g00.imag(), cs[i].g01.real(), cs[i].g01.imag(),
                         cs[i].g10.real(), cs[i].g10.imag(), cs[i].g11.real(), cs[i].g11.imag()};
    for (int q = 0; q < 8; ++q) {
      P.g[q] = (float)v[q];
      P.gl[q] = lo32(v[q]);
    }
    const long long grid = (long long)P.tiles * ((n + P.ppc - 1) / P.ppc);
    cs_site_kernel<<<(int)grid, STAGE_THREADS, 0, st>>>(P);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
  }
  return FFGB_OK;
}

}  // namespace

int stage_rotate_rows(const void* in, void* out, int norb, int nocc, long long ld, long long ncols,
                      const SectorPlan& plan, bool comp, const void* ph_in, const void* ph_out,
                      cudaStream_t st) {
  if (plan.kind != PLAN_CSD) return fail(FFGB_ERR_ARG, "stage path needs a cosine-sine plan");
  if (plan.h < 4 || plan.h > 8 || norb - plan.h < 4 || norb - plan.h > 8)
    return fail(FFGB_ERR_UNSUPPORTED, "stage path needs half windows of 4 to 8 orbitals");
  const HalfTables T = half_tables(norb, nocc, plan.h);
  const float2* src = (const float2*)in;
  float2* dst = (float2*)out;
  FFGB_TRY(window_stage(src, dst, ld, ncols, norb, nocc, T, true, plan.b1, comp, (const float2*)ph_in, nullptr, st));
  FFGB_TRY(window_stage(dst, dst, ld, ncols, norb, nocc, T, false, plan.b2, comp, nullptr, nullptr, st));
  FFGB_TRY(cs_stage(dst, ld, ncols, norb, nocc, plan.h, plan.cs, comp, st));
  FFGB_TRY(window_stage(dst, dst, ld, ncols, norb, nocc, T, true, plan.a1, comp, nullptr, nullptr, st));
  FFGB_TRY(window_stage(dst, dst, ld, ncols, norb, nocc, T, false, plan.a2, comp, nullptr, (const float2*)ph_out, st));
  return FFGB_OK;
}

template <typename T>
int launch_transpose(const void* in, void* out, long long rows, long long cols, const void* row_ph,
                     const void* col_ph, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  if (rows <= 0 || cols <= 0) return FFGB_OK;
  const long long gy = (rows + 31) / 32;
  if (gy > 65535) return fail(FFGB_ERR_UNSUPPORTED, "transpose: too many rows");
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)gy);
  transpose_kernel<Cx><<<grid, 256, 0, st>>>((const Cx*)in, (Cx*)out, rows, cols, (const Cx*)row_ph,
                                             (const Cx*)col_ph);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_transpose<float>(const void*, void*, long long, long long, const void*, const void*,
                                     cudaStream_t);
template int launch_transpose<double>(const void*, void*, long long, long long, const void*, const void*,
                                      cudaStream_t);

template <typename T>
int launch_string_phases(const unsigned* strings, long long dim, int norb, const double* d_host, void* out,
                         cudaStream_t st) {
  using Cx = typename CT<T>::type;
  OrbPhases D;
  std::memset(&D, 0, sizeof(D));
  for (int i = 0; i < 2 * norb && i < 2 * FFGB_MAXN; ++i) D.d[i] = d_host[i];
  string_phase_kernel<Cx><<<(unsigned)((dim + 255) / 256), 256, 0, st>>>(strings, dim, norb, D, (Cx*)out);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_string_phases<float>(const unsigned*, long long, int, const double*, void*, cudaStream_t);
template int launch_string_phases<double>(const unsigned*, long long, int, const double*, void*, cudaStream_t);

template <typename T>
int launch_row_scale(void* x, long long rows, long long ld, const void* ph, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  const long long n = rows * ld;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192));
  row_scale_kernel<Cx><<<blocks, 256, 0, st>>>((Cx*)x, rows, ld, (const Cx*)ph);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_row_scale<float>(void*, long long, long long, const void*, cudaStream_t);
template int launch_row_scale<double>(void*, long long, long long, const void*, cudaStream_t);

template <typename T>
int launch_axpy(const void* x, void* y, long long n, double a, cudaStream_t st) {
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192));
  axpy_kernel<T><<<blocks, 256, 0, st>>>((const typename CT<T>::type*)x, (typename CT<T>::type*)y, n, (T)a,
                                         (T)0);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_axpy<float>(const void*, void*, long long, double, cudaStream_t);
template int launch_axpy<double>(const void*, void*, long long, double, cudaStream_t);

}  // namespace ffgb
