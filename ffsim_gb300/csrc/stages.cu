// Host side of the stage-major complex64 path (see stages.cuh).
#include <algorithm>
#include <cmath>
#include <cstdint>
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

template <int B, int K>
int launch_win_bk(const WinJob& P, int kind, bool low, int epi, long long items, cudaStream_t st,
                  int* grid_used);

namespace {

// Fork/join of a stage's independent launches (its classes touch disjoint
// rows) over auxiliary streams, so that one class's last partial wave
// overlaps the next class instead of leaving SMs idle.  One set of streams and
// events per (device, calling stream), created on first use.
constexpr int FORK_LANES = 3;

struct ForkSet {
  cudaStream_t lane[FORK_LANES] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t done[FORK_LANES] = {};
};

std::mutex g_fork_mu;
std::map<std::pair<int, cudaStream_t>, ForkSet> g_fork;

class StageFork {
 public:
  // n_jobs <= 1 runs everything on the calling stream
  int begin(cudaStream_t main, int n_jobs) {
    main_ = main;
    if (n_jobs <= 1) return FFGB_OK;
    int dev = 0;
    FFGB_CUDA(cudaGetDevice(&dev));
    {
      std::lock_guard<std::mutex> lk(g_fork_mu);
      ForkSet& f = g_fork[std::make_pair(dev, main)];
      if (!f.fork) {
        for (int i = 0; i < FORK_LANES; ++i) {
          FFGB_CUDA(cudaStreamCreateWithFlags(&f.lane[i], cudaStreamNonBlocking));
          FFGB_CUDA(cudaEventCreateWithFlags(&f.done[i], cudaEventDisableTiming));
        }
        FFGB_CUDA(cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming));
      }
      set_ = &f;
    }
    FFGB_CUDA(cudaEventRecord(set_->fork, main));
    for (int i = 0; i < FORK_LANES; ++i) FFGB_CUDA(cudaStreamWaitEvent(set_->lane[i], set_->fork, 0));
    return FFGB_OK;
  }
  cudaStream_t lane(int i) const { return set_ ? set_->lane[i % FORK_LANES] : main_; }
  int end() {
    if (!set_) return FFGB_OK;
    for (int i = 0; i < FORK_LANES; ++i) {
      FFGB_CUDA(cudaEventRecord(set_->done[i], set_->lane[i]));
      FFGB_CUDA(cudaStreamWaitEvent(main_, set_->done[i], 0));
    }
    set_ = nullptr;
    return FFGB_OK;
  }

 private:
  cudaStream_t main_ = nullptr;
  ForkSet* set_ = nullptr;
};

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

int popcount(unsigned x) {
  int c = 0;
  for (; x; x &= x - 1) ++c;
  return c;
}

// Coefficient tables of one rotation list for win_coef<mode>.
void put_coefs(const double* v, int n, int mode, float* gp, float* gl, unsigned* gt) {
  for (int i = 0; i < n; ++i) {
    const double x = v[i];
    if (mode == 2) {
      float dn = (float)x;
      if ((double)dn > x) dn = std::nextafter(dn, -INFINITY);
      const float up = std::nextafter(dn, INFINITY);
      const double p = (x - (double)dn) / ((double)up - (double)dn);
      gp[i] = dn;
      gl[i] = up;
      gt[i] = (unsigned)std::min(4294967295.0, std::max(0.0, std::floor(p * 4294967296.0 + 0.5)));
    } else {
      gp[i] = (float)x;
      gl[i] = (float)(x - (double)(float)x);
      gt[i] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// fused cross-half tables
// ---------------------------------------------------------------------------
// One launch of the cross-half stage: groups with m active sites, their
// tables at `base` (1 + 2^m ints per group).
struct CsClass {
  int m = 0, groups = 0;
  long long base = 0;
  bool sub = false;  // a sub-pass class (ordered: sub-pass A before the B classes)
};

struct CsPass {
  int* tab = nullptr;  // device
  std::vector<CsClass> cls;  // in launch order
};

std::mutex g_cs_mu;
std::map<std::tuple<int, int, int, int, int>, CsPass> g_cs;

// Groups of the sector (norb, nocc) under all cross-half sites i < hh, site i
// rotating orbitals (lo + i, lo + hh + i), for one pass over the state.  Groups
// with at most CS_MAX_M active sites are one class each; a larger group (rare:
// 2% of the rows at norb 16) runs as two sub-passes, first over its first four
// active sites (one sub-group per setting of the others), then over the rest,
// and these classes come last in this order.
int cs_pass_tables(int norb, int nocc, int lo, int hh, const CsPass** out) {
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_cs_mu);
  auto key = std::make_tuple(dev, norb, nocc, lo, hh);
  auto it = g_cs.find(key);
  if (it != g_cs.end()) {
    *out = &it->second;
    return FFGB_OK;
  }
  const long long dim = C(norb, nocc);
  // per class: direct m = 1..CS_MAX_M, then sub-pass A (4 sites), then sub-pass B (m - 4 = 1..4 sites)
  std::vector<std::vector<int>> direct(CS_MAX_M + 1), sub_a(1), sub_b(5);
  std::vector<int> n_direct(CS_MAX_M + 1, 0), n_sub_b(5, 0);
  int n_sub_a = 0;
  // one (sub-)group: base string, its sites (indices into act) and the table entries
  auto emit = [&](std::vector<int>& T, unsigned base, const int* sites, int m) -> int {
    int header = 0;
    for (int t = 0; t < m; ++t) header |= sites[t] << (4 * t);
    T.push_back(header);
    for (int j = 0; j < (1 << m); ++j) {
      unsigned mem = base;
      for (int t = 0; t < m; ++t)
        if ((j >> t) & 1) mem ^= (1u << (lo + sites[t])) | (1u << (lo + hh + sites[t]));
      int sign = 0;
      for (int t = 0; t < m; ++t) {
        if ((j >> t) & 1) continue;
        const int i = lo + sites[t], jj = lo + hh + sites[t];
        const unsigned between = ((1u << jj) - 1u) & ~((1u << (i + 1)) - 1u);
        if (popcount(mem & between) & 1) sign |= 1 << t;
      }
      const long long r = rank(mem);
      if (r >= (1 << 24)) return fail(FFGB_ERR_UNSUPPORTED, "sector too large for the cross-half tables");
      T.push_back((int)r | (sign << 24));
    }
    return FFGB_OK;
  };
  for (long long a = 0; a < dim; ++a) {
    const unsigned s = unrank(a, norb, nocc);
    int act[CS_MAX_SITES], m = 0;
    bool canonical = true;
    for (int i = 0; i < hh; ++i) {
      const bool o_lo = (s >> (lo + i)) & 1u, o_hi = (s >> (lo + hh + i)) & 1u;
      if (o_lo != o_hi) {
        act[m++] = i;
        if (o_hi) canonical = false;  // the group is emitted from its all-low member
      }
    }
    if (m == 0 || !canonical) continue;
    if (m <= CS_MAX_M) {
      FFGB_TRY(emit(direct[m], s, act, m));
      ++n_direct[m];
      continue;
    }
    if (m > 8) return fail(FFGB_ERR_UNSUPPORTED, "too many active cross-half sites");
    const int mb = m - 4;
    auto flip = [&](unsigned x, int t) { return x ^ ((1u << (lo + act[t])) | (1u << (lo + hh + act[t]))); };
    for (int b = 0; b < (1 << mb); ++b) {  // sub-pass A: sites act[0..4), act[4..m) set by b
      unsigned base = s;
      for (int t = 0; t < mb; ++t)
        if ((b >> t) & 1) base = flip(base, 4 + t);
      FFGB_TRY(emit(sub_a[0], base, act, 4));
      ++n_sub_a;
    }
    for (int b = 0; b < 16; ++b) {  // sub-pass B: sites act[4..m), act[0..4) set by b
      unsigned base = s;
      for (int t = 0; t < 4; ++t)
        if ((b >> t) & 1) base = flip(base, t);
      FFGB_TRY(emit(sub_b[mb], base, act + 4, mb));
      ++n_sub_b[mb];
    }
  }
  CsPass P;
  std::vector<int> host;
  auto add = [&](int m, int groups, const std::vector<int>& T, bool sub) {
    if (groups == 0) return;
    CsClass c;
    c.m = m;
    c.groups = groups;
    c.sub = sub;
    c.base = (long long)host.size();
    host.insert(host.end(), T.begin(), T.end());
    P.cls.push_back(c);
  };
  for (int m = CS_MAX_M; m >= 1; --m) add(m, n_direct[m], direct[m], false);
  add(4, n_sub_a, sub_a[0], true);
  for (int m = 4; m >= 1; --m) add(m, n_sub_b[m], sub_b[m], true);
  const size_t bytes = std::max<size_t>(host.size(), 1) * sizeof(int);
  FFGB_CUDA(cudaMalloc(&P.tab, bytes));
  count_alloc();
  if (!host.empty()) FFGB_CUDA(cudaMemcpy(P.tab, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice));
  g_cs[key] = std::move(P);
  *out = &g_cs[key];
  return FFGB_OK;
}

// Groups of 5 and 6 active sites with dithered coefficients run on two lanes
// per column (cs_pair_kernel, 64-column tiles).
template <int M>
int launch_cs_pair(const CsStageParams& P0, long long n_chunks, cudaStream_t st) {
  CsStageParams P = P0;
  P.tiles = (int)((P.ncols + STAGE_THREADS / 2 - 1) / (STAGE_THREADS / 2));
  const long long grid = n_chunks * P.tiles;
  if (grid > 0x7fffffffLL) return fail(FFGB_ERR_UNSUPPORTED, "cross-half stage grid too large");
  cs_pair_kernel<M, 2><<<(unsigned)grid, STAGE_THREADS, 0, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

template <int M>
int launch_cs(const CsStageParams& P, int grid, int mode, cudaStream_t st) {
  if (mode == 0)
    cs_stage_kernel<M, 0><<<grid, STAGE_THREADS, 0, st>>>(P);
  else if (mode == 1)
    cs_stage_kernel<M, 1><<<grid, STAGE_THREADS, 0, st>>>(P);
  else
    cs_stage_kernel<M, 2><<<grid, STAGE_THREADS, 0, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

int cs_stage(float2* x, long long ld, long long ncols, int norb, int nocc, int lo, int hh,
             const std::vector<Pair2>& cs, int mode, unsigned salt, long long col_period, cudaStream_t st) {
  if (hh > CS_MAX_SITES) return fail(FFGB_ERR_UNSUPPORTED, "too many cross-half sites");
  const CsPass* T = nullptr;
  FFGB_TRY(cs_pass_tables(norb, nocc, lo, hh, &T));
  CsStageParams P;
  std::memset(&P, 0, sizeof(P));
  P.x = x;
  P.ld = ld;
  P.ncols = ncols;
  P.tiles = (int)((ncols + STAGE_THREADS - 1) / STAGE_THREADS);
  P.col_period = col_period;
  double v[3 * CS_MAX_SITES] = {};
  for (int i = 0; i < hh; ++i) {
    v[3 * i] = cs[i].g00.real();
    v[3 * i + 1] = cs[i].g01.real();
    v[3 * i + 2] = cs[i].g01.imag();
  }
  put_coefs(v, 3 * CS_MAX_SITES, mode, P.gp, P.gl, P.gt);
  // direct classes round-robin over the fork's lanes; every sub-pass class on
  // the last lane, in order
  StageFork fork;
  FFGB_TRY(fork.begin(st, (int)T->cls.size()));
  int n_direct = 0;
  for (size_t c = 0; c < T->cls.size(); ++c) {
    const CsClass& k = T->cls[c];
    const cudaStream_t ls = fork.lane(k.sub ? FORK_LANES - 1 : n_direct++);
    P.tab = T->tab + k.base;
    P.n_groups = k.groups;
    P.gpc = k.m >= 5 ? CS_MAX_GPC / 2 : CS_MAX_GPC;
    // every launch draws its own dithered coefficients
    P.salt = salt * 0x9E3779B9u + 0x51ED270Bu * (unsigned)(c + 1);
    const long long grid = (long long)((P.n_groups + P.gpc - 1) / P.gpc) * P.tiles;
    if (grid <= 0) continue;
    if (grid > 0x7fffffffLL) return fail(FFGB_ERR_UNSUPPORTED, "cross-half stage grid too large");
    if (mode == 2 && k.m >= 5) {
      const long long n_chunks = (P.n_groups + P.gpc - 1) / P.gpc;
      FFGB_TRY(k.m == 5 ? launch_cs_pair<5>(P, n_chunks, ls) : launch_cs_pair<6>(P, n_chunks, ls));
      continue;
    }
    switch (k.m) {
      case 1: FFGB_TRY(launch_cs<1>(P, (int)grid, mode, ls)); break;
      case 2: FFGB_TRY(launch_cs<2>(P, (int)grid, mode, ls)); break;
      case 3: FFGB_TRY(launch_cs<3>(P, (int)grid, mode, ls)); break;
      case 4: FFGB_TRY(launch_cs<4>(P, (int)grid, mode, ls)); break;
      case 5: FFGB_TRY(launch_cs<5>(P, (int)grid, mode, ls)); break;
      case 6: FFGB_TRY(launch_cs<6>(P, (int)grid, mode, ls)); break;
      default: return fail(FFGB_ERR_ARG, "bad cross-half class");
    }
  }
  return fork.end();
}

template <int B, int K = 0>
int launch_job_k(int k, const WinJob& P, int kind, bool low, int epi, long long items, cudaStream_t st,
                 int* grid_used) {
  if constexpr (K <= B) {
    if (k == K) return launch_win_bk<B, K>(P, kind, low, epi, items, st, grid_used);
    return launch_job_k<B, K + 1>(k, P, kind, low, epi, items, st, grid_used);
  } else {
    return fail(FFGB_ERR_ARG, "window class out of range");
  }
}

int launch_job_b(int b, const WinJob& P, int k, int kind, bool low, int epi, long long items,
                 cudaStream_t st, int* grid_used) {
  switch (b) {
    case 4: return launch_job_k<4>(k, P, kind, low, epi, items, st, grid_used);
    case 5: return launch_job_k<5>(k, P, kind, low, epi, items, st, grid_used);
    case 6: return launch_job_k<6>(k, P, kind, low, epi, items, st, grid_used);
    case 7: return launch_job_k<7>(k, P, kind, low, epi, items, st, grid_used);
    case 8: return launch_job_k<8>(k, P, kind, low, epi, items, st, grid_used);
    default: return fail(FFGB_ERR_UNSUPPORTED, "window size outside [4, 8]");
  }
}

// Layout of a window [lo, lo + B) of the sector (norb, nocc): one class per
// (k electrons inside, m0 electrons below lo).  A group of a class fixes the
// occupation outside the window; its member j (colex order of the window
// pattern w_j) sits at row base[g] + off[j] with
//   base[g] = rank(below) + rank_shifted(above, lo + B, m0 + k),
//   off[j]  = rank_shifted(w_j, lo, m0).
struct WinClass {
  int k, m0;
  long long groups;
  long long base_off;  // first entry of this class in the device base table
  std::vector<int> off;
};
struct WinLayout {
  std::vector<WinClass> cls;
  int* dev_base = nullptr;
};

std::mutex g_win_mu;
std::map<std::tuple<int, int, int, int, int>, WinLayout> g_win;

int win_layout(int norb, int nocc, int lo, int B, const WinLayout** out) {
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_win_mu);
  auto key = std::make_tuple(dev, norb, nocc, lo, B);
  auto it = g_win.find(key);
  if (it != g_win.end()) {
    *out = &it->second;
    return FFGB_OK;
  }
  const int above = norb - lo - B;
  WinLayout W;
  std::vector<int> host;
  for (int k = std::max(0, nocc - lo - above); k <= std::min(B, nocc); ++k)
    for (int m0 = std::max(0, nocc - k - above); m0 <= std::min(lo, nocc - k); ++m0) {
      WinClass c;
      c.k = k;
      c.m0 = m0;
      const int ma = nocc - k - m0;
      c.base_off = (long long)host.size();
      for (long long ib = 0; ib < C(lo, m0); ++ib) {
        const long long rb = rank(unrank(ib, lo, m0));
        for (long long ia = 0; ia < C(above, ma); ++ia) {
          const long long r = rb + rank_shifted(unrank(ia, above, ma), lo + B, m0 + k);
          if (r >= (1LL << 31)) return fail(FFGB_ERR_UNSUPPORTED, "sector too large");
          host.push_back((int)r);
        }
      }
      c.groups = (long long)host.size() - c.base_off;
      for (long long j = 0; j < C(B, k); ++j) c.off.push_back((int)rank_shifted(unrank(j, B, k), lo, m0));
      if (c.groups > 0) W.cls.push_back(std::move(c));
    }
  const size_t bytes = std::max<size_t>(host.size(), 1) * sizeof(int);
  FFGB_CUDA(cudaMalloc(&W.dev_base, bytes));
  count_alloc();
  if (!host.empty())
    FFGB_CUDA(cudaMemcpy(W.dev_base, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice));
  g_win[key] = std::move(W);
  *out = &g_win[key];
  return FFGB_OK;
}

// One window stage on [lo, lo + B).  Every class is one launch; classes k and
// B - k with the same m0 are processed together (complement-packed) where
// their registers fit, and k = B/2 is packed within its groups.
int window_stage(const float2* in, float2* out, long long ld, long long ncols, int norb, int nocc, int lo, int B,
                 const std::vector<Givens>& net, unsigned salt, const StageExpectArgs* ex, int* ex_ctas,
                 long long col_period, cudaStream_t st) {
  if (B < 4 || B > 8) return fail(FFGB_ERR_UNSUPPORTED, "window size outside [4, 8]");
  const WinLayout* L = nullptr;
  FFGB_TRY(win_layout(norb, nocc, lo, B, &L));
  const bool low = lo == 0;  // members are consecutive rows
  auto base = std::make_unique<WinJob>();
  std::memset(base.get(), 0, sizeof(WinJob));
  base->in = in;
  base->out = out;
  base->ld = ld;
  base->ncols = ncols;
  base->tiles = (int)((ncols + STAGE_THREADS - 1) / STAGE_THREADS);
  base->norb = norb;
  base->lo = lo;
  base->salt = salt;
  base->col_period = col_period;
  const int epi = ex ? EPI_EXPECT : EPI_STORE;
  std::vector<double> v(3 * net.size());
  for (size_t g = 0; g < net.size(); ++g) {
    v[3 * g] = net[g].c;
    v[3 * g + 1] = net[g].s.real();
    v[3 * g + 2] = net[g].s.imag();
  }
  if (v.size() > 84) return fail(FFGB_ERR_UNSUPPORTED, "window network too long");
  put_coefs(v.data(), (int)v.size(), 2, base->gp, base->gl, base->gt);
  if (ex) {
    StageExpect& E = base->ex;
    E.zrow = ex->zrow;
    E.zcol = ex->zcol;
    E.row_str = ex->row_str;
    E.col_str = ex->col_str;
    E.zrep = ex->zrep;
    E.col_period = ex->col_period;
    E.col_valid = ex->col_valid;
    for (int i = 0; i < FFGB_MAXN; ++i)
      for (int l = 0; l < FFGB_MAXN; ++l) {
        E.X[i][l] = ex->X[i][l];
        E.Xsum[l] += ex->X[i][l];
      }
  }
  struct Job {
    const WinClass *a, *b;
    int kind;
    long long n, start, work;
  };
  auto find = [&](int k, int m0) -> const WinClass* {
    for (const WinClass& c : L->cls)
      if (c.k == k && c.m0 == m0) return &c;
    return nullptr;
  };
  std::vector<Job> jobs;
  for (const WinClass& c : L->cls) {
    const int kp = B - c.k;
    const WinClass* partner = find(kp, c.m0);
    const bool packable = 2 * c.k < B && C(B, c.k) <= 35;
    const bool partner_packs = 2 * c.k > B && C(B, kp) <= 35 && partner;
    if (partner_packs) continue;  // taken with its partner
    if (2 * c.k == B) {
      // packed within the group on windows starting at orbital 0; elsewhere the
      // member-offset table pushes the packed kernel into spills
      jobs.push_back({&c, nullptr, low ? 1 : 0, c.groups, 0, c.groups * C(B, c.k)});
    } else if (packable && partner) {
      const long long np = std::min(c.groups, partner->groups);
      jobs.push_back({&c, partner, 2, np, 0, 2 * np * C(B, c.k)});
      if (c.groups > np) jobs.push_back({&c, nullptr, 0, c.groups - np, np, (c.groups - np) * C(B, c.k)});
      if (partner->groups > np)
        jobs.push_back({partner, nullptr, 0, partner->groups - np, np, (partner->groups - np) * C(B, kp)});
    } else {
      jobs.push_back({&c, nullptr, 0, c.groups, 0, c.groups * C(B, c.k)});
    }
  }
  std::stable_sort(jobs.begin(), jobs.end(), [](const Job& x, const Job& y) { return x.work > y.work; });
  long long pbase = 0;
  WinJob P;
  // the jobs touch disjoint rows (and disjoint partial sums): forked over lanes
  StageFork fork;
  FFGB_TRY(fork.begin(st, (int)jobs.size()));
  int lane = 0;
  for (const Job& jb : jobs) {
    std::memcpy(&P, base.get(), sizeof(WinJob));
    if (jb.a->off.size() > 72) return fail(FFGB_ERR_UNSUPPORTED, "window member table overflow");
    P.gbase_a = L->dev_base + jb.a->base_off + jb.start;
    for (size_t j = 0; j < jb.a->off.size(); ++j) {
      P.off_a[j] = jb.a->off[j];
      P.eoff_a[j] = (long long)jb.a->off[j] * ld;
    }
    if (jb.b) {
      P.gbase_b = L->dev_base + jb.b->base_off;
      for (size_t j = 0; j < jb.b->off.size(); ++j) {
        P.off_b[j] = jb.b->off[j];
        P.eoff_b[j] = (long long)jb.b->off[j] * ld;
      }
    }
    P.n_groups = (int)jb.n;
    const long long items = jb.n * base->tiles;
    if (items <= 0) continue;
    if (items > 0x7fffffffLL) return fail(FFGB_ERR_UNSUPPORTED, "window stage grid too large");
    if (ex) {
      if (pbase + items > ex->partial_cap) return fail(FFGB_ERR_OOM, "partial-sum buffer too small");
      P.ex.partials = ex->partials + pbase;
    }
    int used = 0;
    FFGB_TRY(launch_job_b(B, P, jb.a->k, jb.kind, low, epi, items, fork.lane(lane++), &used));
    pbase += used;
  }
  FFGB_TRY(fork.end());
  if (ex_ctas) *ex_ctas = (int)pbase;
  return FFGB_OK;
}

}  // namespace

static_assert(STACK_TILE == STAGE_THREADS, "stacked states are padded to the stage kernels' column tile");

long long stage_expect_partials(long long rows, long long ncols) {
  return std::max<long long>(rows, 1) * ((ncols + STAGE_THREADS - 1) / STAGE_THREADS);
}

int stage_rotate_rows(const void* in, void* out, int norb, int nocc, long long ld, long long ncols,
                      const SectorPlan& plan, const StageOpts& o, cudaStream_t st) {
  if (plan.kind != PLAN_CSD || plan.ops.empty()) return fail(FFGB_ERR_ARG, "stage path needs a cosine-sine plan");
  if (o.mode != 2) return fail(FFGB_ERR_ARG, "stage kernels use dithered coefficients");
  const int n_ops = (int)plan.ops.size();
  if (plan.ops[0].type != 0 || plan.ops[n_ops - 1].type != 0)
    return fail(FFGB_ERR_ARG, "a cosine-sine plan starts and ends with window stages");
  const unsigned s = o.salt * 0x2545F491u;
  int first = 0, last = n_ops - 1;
  if (o.only_stage >= 0) {
    if (o.only_stage >= n_ops) return fail(FFGB_ERR_ARG, "stage index out of range");
    if (plan.ops[o.only_stage].type == 1 && in != out) return fail(FFGB_ERR_ARG, "the cross-half stage runs in place");
    first = last = o.only_stage;
  }
  for (int i = first; i <= last; ++i) {
    const StageOp& op = plan.ops[i];
    const float2* src = (const float2*)(i == first ? in : out);
    float2* dst = (float2*)out;
    if (op.type == 0) {
      const bool fused = o.expect && i == n_ops - 1 && o.only_stage < 0;
      FFGB_TRY(window_stage(src, dst, ld, ncols, norb, nocc, op.lo, op.b, op.net, s + 1 + i,
                            fused ? o.expect : nullptr, fused ? o.expect_ctas : nullptr, o.col_period, st));
    } else {
      FFGB_TRY(cs_stage(dst, ld, ncols, norb, nocc, op.lo, op.b, op.pairs, o.mode, s + 1 + i, o.col_period, st));
    }
  }
  return FFGB_OK;
}

template <typename T>
int launch_transpose(const void* in, void* out, long long rows, long long cols, const void* row_ph,
                     const void* col_ph, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  if (rows <= 0 || cols <= 0) return FFGB_OK;
  const long long gy = (rows + 63) / 64;
  if (gy > 65535) return fail(FFGB_ERR_UNSUPPORTED, "transpose: too many rows");
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)gy);
  transpose_kernel<Cx><<<grid, 256, 0, st>>>((const Cx*)in, (Cx*)out, rows, cols, cols, rows, 0, 0,
                                             (const Cx*)row_ph, (const Cx*)col_ph);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_transpose<float>(const void*, void*, long long, long long, const void*, const void*,
                                     cudaStream_t);

template <typename T>
int launch_transpose_stacked(const void* in, void* out, long long rows, long long cols, long long n_states,
                             long long in_pad, long long out_pad, const void* row_ph, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  if (rows <= 0 || cols <= 0 || n_states <= 0) return FFGB_OK;
  const long long gy = (rows + 63) / 64;
  if (gy > 65535 || n_states > 65535) return fail(FFGB_ERR_UNSUPPORTED, "stacked transpose: grid too large");
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)gy, (unsigned)n_states);
  transpose_kernel<Cx><<<grid, 256, 0, st>>>((const Cx*)in, (Cx*)out, rows, cols, n_states * in_pad,
                                             n_states * out_pad, in_pad, out_pad, (const Cx*)row_ph, nullptr);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_transpose_stacked<float>(const void*, void*, long long, long long, long long, long long,
                                             long long, const void*, cudaStream_t);
template int launch_transpose_stacked<double>(const void*, void*, long long, long long, long long, long long,
                                              long long, const void*, cudaStream_t);

template <typename T>
int launch_stack(void* x, void* y, long long n_states, long long rows, long long cols, long long pad, int dir,
                 int accumulate, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  const long long n = n_states * rows * cols;
  if (n <= 0) return FFGB_OK;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192));
  stack_kernel<Cx><<<blocks, 256, 0, st>>>((Cx*)x, (Cx*)y, n_states, rows, cols, pad, dir, accumulate);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_stack<float>(void*, void*, long long, long long, long long, long long, int, int, cudaStream_t);
template int launch_stack<double>(void*, void*, long long, long long, long long, long long, int, int, cudaStream_t);

int launch_state_partials(const double* partials, long long n, long long tiles, long long tiles_per_state,
                          long long n_states, double* out, cudaStream_t st) {
  if (n_states <= 0) return FFGB_OK;
  if (n_states > 0x7fffffffLL) return fail(FFGB_ERR_UNSUPPORTED, "too many states");
  state_partials_kernel<<<(unsigned)n_states, 256, 0, st>>>(partials, n, tiles, tiles_per_state, out);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
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
int launch_row_axpy(const void* x, void* y, long long rows, long long ld, const void* ph, cudaStream_t st) {
  using Cx = typename CT<T>::type;
  const long long n = rows * ld;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192));
  row_axpy_kernel<Cx><<<blocks, 256, 0, st>>>((const Cx*)x, (Cx*)y, rows, ld, (const Cx*)ph);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}
template int launch_row_axpy<float>(const void*, void*, long long, long long, const void*, cudaStream_t);
template int launch_row_axpy<double>(const void*, void*, long long, long long, const void*, cudaStream_t);

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
