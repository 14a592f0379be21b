// Resident evaluator: a persistent kernel that evaluates LUCJ energies of
// small shapes (norb <= 8, any nelec, complex64 state, FP64 energy) taken
// from a work queue in host-mapped memory.
//
// The batch path launches a few hundred kernels per evaluation; at norb 8 a
// state is 4,900 amplitudes, so those launches, not the work, set its cost.
// Here one CTA evaluates one request end to end with the state in shared
// memory: the UCJ circuit from Hartree-Fock, then every term of the
// request's double-factorized Hamiltonian, and writes the energy back to the
// request's slot.  Requests of different shapes and Hamiltonians share one
// queue and one kernel.
//
// Queue protocol (host: ffgb_resident_*; device: resident_kernel):
//  * the host writes a job into slot (ticket mod n_slots), marks it READY and
//    then publishes it by advancing `head` (release store);
//  * thread 0 of a CTA claims the next ticket with a compare-and-swap on the
//    device counter `tail`, only below `head` (acquire load), so a claimed
//    ticket always has its job written;
//  * the CTA copies the job into shared memory, evaluates it (reading the
//    slot's cancel word between gates), writes energy and status, and marks
//    the slot DONE (release store);
//  * the wait for work is bounded: a CTA that finds no work for `idle_ns`
//    (globaltimer) or after a fixed number of polls exits, and the last CTA
//    to exit records FFGB_ERR_TIMEOUT as the kernel's status; `stop` makes
//    every CTA exit between jobs with FFGB_OK.  The host relaunches the kernel
//    when it has exited and work is waiting.
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.h"
#include "plan.h"

namespace ffgb {
namespace {

constexpr int RES_MAXN = 8;
constexpr int RES_MAX_REPS = 4;
constexpr int RES_MAXDIM = 70;  // C(8, 4)
constexpr int RES_THREADS = 128;
constexpr int RES_NET = 28 * 3;  // (c, Re s, Im s) of the 28 rotations of an 8-orbital brick network
constexpr int RES_MAX_TERMS = 4096;

enum { RES_FREE = 0, RES_READY = 1, RES_DONE = 2 };

// W(V) on both spin sectors: V's brick network (plan_sector, FULL kind),
// compensated FP32 coefficients, then the orbital phases exp(i ang).
struct ResRot {
  float gp[RES_NET];
  float gl[RES_NET];
  double ang[RES_MAXN];
};

// Diagonal operator f(a, b) = sum_{i<=j} A_ij g_i(a) g_j(a)
//   + sum_{i<=j} B_ij g_i(b) g_j(b) + sum_{i,j} X_ij g_i(a) g_j(b),
// g = n (number representation) or 1 - 2n (Z representation).
struct ResDiag {
  double A[RES_MAXN][RES_MAXN];
  double B[RES_MAXN][RES_MAXN];
  double X[RES_MAXN][RES_MAXN];
  int zrep, pad;
};

// A Hamiltonian in device memory: n_terms (U_t, Z_t) pairs; rot holds the
// plans of U_t^dagger (the state is rotated into the term's basis), rot_u
// those of U_t (the matvec of a gradient rotates back).
struct ResHam {
  int norb, n_terms;
  double constant;
  const ResRot* rot;
  const ResRot* rot_u;
  const ResDiag* z;
};

// One request.  Gates: rot[0], diag[0], rot[1], ..., diag[n_reps-1], rot[n_reps];
// the diag gates are exp(i f) phases.  A gradient request (grad != 0) also
// carries the inverse rotations rot_inv[k] (of rot[k]) for its backward pass.
struct alignas(16) ResJob {
  int norb, na, nb, n_reps;
  const ResHam* ham;
  int grad, pad[3];
  ResRot rot[RES_MAX_REPS + 1];
  ResRot rot_inv[RES_MAX_REPS + 1];
  ResDiag diag[RES_MAX_REPS];
};

// Densities of a gradient request, per gate j = 1 .. n_reps + 1 (index j - 1):
// the transition one-body densities <lambda| a+_p a_q |psi> of both sectors
// and the pair densities <lambda| n_i n_j |psi> (aa, ab, bb; gates j >= 2),
// norb x norb each (row stride RES_MAXN).
constexpr int RES_DENS_BLOCKS = 5;

struct alignas(64) ResSlot {
  ResJob job;
  int state;   // RES_FREE / RES_READY (host) / RES_DONE (device)
  int cancel;  // nonzero: the host asks the device to stop this job
  int status;  // FFGB_OK or FFGB_ERR_CANCELLED (device)
  int pad;
  double energy;
  double2 dens[RES_MAX_REPS + 1][RES_DENS_BLOCKS][RES_MAXN * RES_MAXN];
};

struct ResQueue {  // host-mapped
  unsigned long long head;  // tickets published
  int stop;                 // nonzero: every CTA exits between jobs
  int kstatus;              // exit status of the last kernel (set by its last CTA)
};

struct ResDev {  // device memory
  unsigned long long tail;  // tickets claimed
  int running;              // CTAs alive
  int pad;
  float2* lam;              // per CTA one state (the gradient's lambda), RES_MAXDIM^2 amplitudes
};

static_assert(sizeof(ResJob) % 16 == 0, "jobs are copied in 16-byte words");

// --- system-scope accesses to host-mapped memory ---------------------------
__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_sys(const int* p) {
  int v;
  asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(int* p, int v) {
  asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Claim the next ticket (thread 0).  >= 0: the ticket; -1: stop requested;
// -2: no work within idle_ns (or the poll limit).
__device__ long long res_claim(ResQueue* q, ResDev* d, unsigned long long idle_ns) {
  const unsigned long long t0 = globaltimer_ns();
  const long long max_polls = (long long)(idle_ns / 2000ull) * 4 + 1024;
  for (long long it = 0; it < max_polls; ++it) {
    if (ld_relaxed_sys(&q->stop)) return -1;
    const unsigned long long h = ld_acquire_sys(&q->head);
    const unsigned long long c = atomicAdd(&d->tail, 0ull);
    if (c < h) {
      if (atomicCAS(&d->tail, c, c + 1) == c) return (long long)c;
      continue;  // another CTA took it
    }
    if (globaltimer_ns() - t0 > idle_ns) return -2;
    __nanosleep(2000);
  }
  return -2;
}

__device__ __forceinline__ float res_g(unsigned s, int i, int zrep) {
  const unsigned b = (s >> i) & 1u;
  return zrep ? (b ? -1.f : 1.f) : (float)b;
}
__device__ __forceinline__ double res_gd(unsigned s, int i, int zrep) {
  const unsigned b = (s >> i) & 1u;
  return zrep ? (b ? -1.0 : 1.0) : (double)b;
}

// sum_{i<=j} M_ij g_i(s) g_j(s) in FP64
__device__ double res_same(const double (&M)[RES_MAXN][RES_MAXN], unsigned s, int n, int zrep) {
  double f = 0.0;
  for (int i = 0; i < n; ++i) {
    const double gi = res_gd(s, i, zrep);
    if (gi == 0.0) continue;
    for (int j = i; j < n; ++j) f += M[i][j] * gi * res_gd(s, j, zrep);
  }
  return f;
}

// Both sectors' networks of one rotation, in place on X (da x db, row-major).
template <int N>
__device__ void res_networks(float2* X, int na, int nb, int da, int db, const int* offa, const int* offb,
                             const float* gp, const float* gl) {
  for (int c = threadIdx.x; c < db; c += RES_THREADS) WinDispatch<N>::template group<true>(na, X + c, offa, gp, gl);
  __syncthreads();
  for (int r = threadIdx.x; r < da; r += RES_THREADS)
    WinDispatch<N>::template group<true>(nb, X + (long long)r * db, offb, gp, gl);
  __syncthreads();
}

__device__ void res_rotate(float2* X, int norb, int na, int nb, int da, int db, const int* offa, const int* offb,
                           const ResRot& R) {
  switch (norb) {
    case 1: res_networks<1>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 2: res_networks<2>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 3: res_networks<3>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 4: res_networks<4>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 5: res_networks<5>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 6: res_networks<6>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 7: res_networks<7>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    case 8: res_networks<8>(X, na, nb, da, db, offa, offb, R.gp, R.gl); break;
    default: break;
  }
}

struct ResTables {
  unsigned sa[RES_MAXDIM], sb[RES_MAXDIM];  // strings of both sectors (colex order)
  int offa[RES_MAXDIM], offb[RES_MAXDIM];   // member offsets: alpha down a column, beta along a row
  double fa[RES_MAXDIM], fb[RES_MAXDIM];    // per-string FP64 parts of a phase
  double wa[RES_MAXDIM][RES_MAXN];          // per alpha string: sum_i X_ij g_i(a)
  float za[RES_MAXDIM], zb[RES_MAXDIM];     // per-string FP32 parts of an expectation
  float wz[RES_MAXDIM][RES_MAXN];
  double red[RES_THREADS / 32];
  short ra[256], rb[256];  // index of a string (bitmask) in each sector, -1 if absent
  ResRot trot;  // the current Hamiltonian term's plan
};

// X *= exp(i (f(a, b) + sum_{i in a} ang_i + sum_{i in b} ang_i)) (f in FP64,
// rounded once per amplitude).  D = NULL: the orbital phases alone.
__device__ void res_phase(float2* X, int norb, int da, int db, const ResDiag* D, const double* ang, ResTables& T,
                          double sign = 1.0) {
  const int zrep = D ? D->zrep : 0;
  for (int s = threadIdx.x; s < da + db; s += RES_THREADS) {
    const bool alpha = s < da;
    const unsigned str = alpha ? T.sa[s] : T.sb[s - da];
    double f = 0.0;
    if (ang)
      for (int i = 0; i < norb; ++i)
        if ((str >> i) & 1u) f += ang[i];
    if (D) f += sign * res_same(alpha ? D->A : D->B, str, norb, zrep);
    if (alpha) {
      T.fa[s] = f;
      for (int j = 0; j < norb; ++j) {
        double w = 0.0;
        if (D)
          for (int i = 0; i < norb; ++i) w += D->X[i][j] * res_gd(str, i, zrep);
        T.wa[s][j] = sign * w;
      }
    } else {
      T.fb[s - da] = f;
    }
  }
  __syncthreads();
  const int n = da * db;
  for (int e = threadIdx.x; e < n; e += RES_THREADS) {
    const int a = e / db, b = e - a * db;
    double f = T.fa[a] + T.fb[b];
    if (D) {
      const unsigned sb = T.sb[b];
      for (int j = 0; j < norb; ++j) f += T.wa[a][j] * res_gd(sb, j, zrep);
    }
    const float2 p = phase_of(f, (float2*)nullptr);
    const float2 x = X[e];
    X[e] = make_float2(x.x * p.x - x.y * p.y, x.x * p.y + x.y * p.x);
  }
  __syncthreads();
}

// Sum over the CTA of one FP64 value per thread, in a fixed order (every
// thread gets the sum).
__device__ double res_block_sum(double acc, ResTables& T) {
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) T.red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < RES_THREADS / 32; ++w) s += T.red[w];
  __syncthreads();
  return s;
}

// Per-string FP32 parts of a diagonal operator (za, zb, wz), FP64 rounded once.
__device__ void res_ztables(int norb, int da, int db, const ResDiag& D, ResTables& T) {
  const int zrep = D.zrep;
  for (int s = threadIdx.x; s < da + db; s += RES_THREADS) {
    const bool alpha = s < da;
    const unsigned str = alpha ? T.sa[s] : T.sb[s - da];
    const double f = res_same(alpha ? D.A : D.B, str, norb, zrep);
    if (alpha) {
      T.za[s] = (float)f;
      for (int j = 0; j < norb; ++j) {
        double w = 0.0;
        for (int i = 0; i < norb; ++i) w += D.X[i][j] * res_gd(str, i, zrep);
        T.wz[s][j] = (float)w;
      }
    } else {
      T.zb[s - da] = (float)f;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float res_z(int norb, int a, int b, int zrep, const ResTables& T) {
  const unsigned sb = T.sb[b];
  float z = T.za[a] + T.zb[b];
  for (int j = 0; j < norb; ++j) z = fmaf(T.wz[a][j], res_g(sb, j, zrep), z);
  return z;
}

// X *= z(a, b) (the coefficient of a diagonal operator).
__device__ void res_coef(float2* X, int norb, int da, int db, const ResDiag& D, ResTables& T) {
  res_ztables(norb, da, db, D, T);
  for (int e = threadIdx.x; e < da * db; e += RES_THREADS) {
    const int a = e / db, b = e - a * db;
    const float z = res_z(norb, a, b, D.zrep, T);
    X[e] = make_float2(z * X[e].x, z * X[e].y);
  }
  __syncthreads();
}

// Transition one-body densities <y| a+_p a_q |x> of both sectors into
// out[0] (alpha) and out[1] (beta), row stride RES_MAXN: one thread per
// (sector, p, q), the strings in order, each string's products summed in
// FP32 and the strings in FP64.
__device__ void res_trdm1(const float2* y, const float2* x, int norb, int da, int db, ResTables& T,
                          double2 (*out)[RES_MAXN * RES_MAXN]) {
  const int n2 = norb * norb;
  for (int t = threadIdx.x; t < 2 * n2; t += RES_THREADS) {
    const int sec = t / n2, pq = t - sec * n2, p = pq / norb, q = pq - p * norb;
    const int dr = sec == 0 ? da : db;
    const unsigned* str = sec == 0 ? T.sa : T.sb;
    const short* rk = sec == 0 ? T.ra : T.rb;
    double ax = 0.0, ay = 0.0;
    for (int r = 0; r < dr; ++r) {
      const unsigned s = str[r];
      if (!((s >> q) & 1u)) continue;
      unsigned t2 = s;
      int sign = 0;
      if (p != q) {
        if ((s >> p) & 1u) continue;
        const unsigned r1 = s & ~(1u << q);
        sign = (__popc(s & ((1u << q) - 1u)) + __popc(r1 & ((1u << p) - 1u))) & 1;
        t2 = r1 | (1u << p);
      }
      const int r2 = rk[t2];
      float2 acc = make_float2(0.f, 0.f);
      if (sec == 0) {
        const float2* yr = y + (long long)r2 * db;
        const float2* xr = x + (long long)r * db;
        for (int c = 0; c < db; ++c) {
          acc.x = fmaf(yr[c].x, xr[c].x, fmaf(yr[c].y, xr[c].y, acc.x));
          acc.y = fmaf(yr[c].x, xr[c].y, fmaf(-yr[c].y, xr[c].x, acc.y));
        }
      } else {
        for (int c = 0; c < da; ++c) {
          const float2 yv = y[(long long)c * db + r2], xv = x[(long long)c * db + r];
          acc.x = fmaf(yv.x, xv.x, fmaf(yv.y, xv.y, acc.x));
          acc.y = fmaf(yv.x, xv.y, fmaf(-yv.y, xv.x, acc.y));
        }
      }
      ax += sign ? -(double)acc.x : (double)acc.x;
      ay += sign ? -(double)acc.y : (double)acc.y;
    }
    out[sec][p * RES_MAXN + q] = make_double2(ax, ay);
  }
}

// Pair densities <y| n_is n_jt |x> for (s, t) = (a, a), (a, b), (b, b) into
// out[0..2] (row stride RES_MAXN).  w = conj(y) x per amplitude; per alpha
// string its row sum and its sums per occupied beta orbital, per beta string
// its column sum (FP32 within a row or column, FP64 after), in `work`
// (RES_MAXDIM * (RES_MAXN + 2) double2); then one thread per entry, strings
// in order.
__device__ void res_pair(const float2* y, const float2* x, int norb, int da, int db, ResTables& T, double2* work,
                         double2 (*out)[RES_MAXN * RES_MAXN]) {
  double2* rsum = work;                      // [da]
  double2* csum = work + RES_MAXDIM;         // [db]
  double2* m = work + 2 * RES_MAXDIM;        // [da][RES_MAXN]
  for (int t = threadIdx.x; t < da + db; t += RES_THREADS) {
    if (t < da) {
      float2 rs = make_float2(0.f, 0.f);
      float2 mj[RES_MAXN];
      for (int j = 0; j < RES_MAXN; ++j) mj[j] = make_float2(0.f, 0.f);
      for (int c = 0; c < db; ++c) {
        const float2 yv = y[(long long)t * db + c], xv = x[(long long)t * db + c];
        const float2 w = make_float2(yv.x * xv.x + yv.y * xv.y, yv.x * xv.y - yv.y * xv.x);
        rs.x += w.x;
        rs.y += w.y;
        const unsigned sb = T.sb[c];
        for (int j = 0; j < norb; ++j)
          if ((sb >> j) & 1u) {
            mj[j].x += w.x;
            mj[j].y += w.y;
          }
      }
      rsum[t] = make_double2(rs.x, rs.y);
      for (int j = 0; j < RES_MAXN; ++j) m[t * RES_MAXN + j] = make_double2(mj[j].x, mj[j].y);
    } else {
      const int c = t - da;
      float2 cs = make_float2(0.f, 0.f);
      for (int r = 0; r < da; ++r) {
        const float2 yv = y[(long long)r * db + c], xv = x[(long long)r * db + c];
        cs.x += yv.x * xv.x + yv.y * xv.y;
        cs.y += yv.x * xv.y - yv.y * xv.x;
      }
      csum[c] = make_double2(cs.x, cs.y);
    }
  }
  __syncthreads();
  const int n2 = norb * norb;
  for (int t = threadIdx.x; t < 3 * n2; t += RES_THREADS) {
    const int blk = t / n2, ij = t - blk * n2, i = ij / norb, j = ij - i * norb;
    double ax = 0.0, ay = 0.0;
    if (blk == 0) {
      for (int r = 0; r < da; ++r)
        if (((T.sa[r] >> i) & 1u) && ((T.sa[r] >> j) & 1u)) {
          ax += rsum[r].x;
          ay += rsum[r].y;
        }
    } else if (blk == 1) {
      for (int r = 0; r < da; ++r)
        if ((T.sa[r] >> i) & 1u) {
          ax += m[r * RES_MAXN + j].x;
          ay += m[r * RES_MAXN + j].y;
        }
    } else {
      for (int c = 0; c < db; ++c)
        if (((T.sb[c] >> i) & 1u) && ((T.sb[c] >> j) & 1u)) {
          ax += csum[c].x;
          ay += csum[c].y;
        }
    }
    out[2 + blk][i * RES_MAXN + j] = make_double2(ax, ay);
  }
  __syncthreads();
}

// sum_{a,b} z(a, b) |X(a, b)|^2: z in FP32 from per-string parts (FP64,
// rounded once), products summed in FP64; the CTA sum in a fixed order.
__device__ double res_expect(const float2* X, int norb, int da, int db, const ResDiag& D, ResTables& T) {
  const int zrep = D.zrep;
  for (int s = threadIdx.x; s < da + db; s += RES_THREADS) {
    const bool alpha = s < da;
    const unsigned str = alpha ? T.sa[s] : T.sb[s - da];
    const double f = res_same(alpha ? D.A : D.B, str, norb, zrep);
    if (alpha) {
      T.za[s] = (float)f;
      for (int j = 0; j < norb; ++j) {
        double w = 0.0;
        for (int i = 0; i < norb; ++i) w += D.X[i][j] * res_gd(str, i, zrep);
        T.wz[s][j] = (float)w;
      }
    } else {
      T.zb[s - da] = (float)f;
    }
  }
  __syncthreads();
  double acc = 0.0;
  const int n = da * db;
  for (int e = threadIdx.x; e < n; e += RES_THREADS) {
    const int a = e / db, b = e - a * db;
    const unsigned sb = T.sb[b];
    float z = T.za[a] + T.zb[b];
    for (int j = 0; j < norb; ++j) z = fmaf(T.wz[a][j], res_g(sb, j, zrep), z);
    const float2 x = X[e];
    acc = fma((double)z, (double)(x.x * x.x + x.y * x.y), acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) T.red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < RES_THREADS / 32; ++w) s += T.red[w];
  __syncthreads();
  return s;
}

// Cancel word of the current slot, read by thread 0 and shared with the CTA.
__device__ bool res_cancelled(ResSlot* S, int* flag) {
  if (threadIdx.x == 0) *flag = ld_relaxed_sys(&S->cancel);
  __syncthreads();
  const bool c = *flag != 0;
  __syncthreads();
  return c;
}

__device__ void res_load_rot(const ResRot* src, ResRot& dst) {
  const float* a = reinterpret_cast<const float*>(src);
  float* b = reinterpret_cast<float*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(ResRot) / 4); i += RES_THREADS) b[i] = a[i];
  __syncthreads();
}

// The adjoint gradient's device part, after the forward circuit left psi:
// lambda = (H - c) psi (every term: rotate by U_t^dag, multiply by z_t,
// rotate by U_t, accumulate), E = c + Re <psi|lambda>, then the gates undone
// on psi and lambda from the last, with the densities of each gate written
// to the slot (the host applies the chain rule).
__device__ int res_gradient(const ResJob& J, ResSlot* S, float2* psi, float2* phi, float2* lam, int da, int db,
                            ResTables& T, int* flag, double* energy) {
  const int norb = J.norb, na = J.na, nb = J.nb, n = da * db;
  const ResHam* H = J.ham;
  for (int e = threadIdx.x; e < n; e += RES_THREADS) lam[e] = make_float2(0.f, 0.f);
  __syncthreads();
  for (int t = 0; t < H->n_terms; ++t) {
    if ((t & 3) == 0 && res_cancelled(S, flag)) return FFGB_ERR_CANCELLED;
    for (int e = threadIdx.x; e < n; e += RES_THREADS) phi[e] = psi[e];
    res_load_rot(H->rot + t, T.trot);
    res_rotate(phi, norb, na, nb, da, db, T.offa, T.offb, T.trot);
    res_phase(phi, norb, da, db, nullptr, T.trot.ang, T);
    res_coef(phi, norb, da, db, H->z[t], T);
    res_load_rot(H->rot_u + t, T.trot);
    res_rotate(phi, norb, na, nb, da, db, T.offa, T.offb, T.trot);
    res_phase(phi, norb, da, db, nullptr, T.trot.ang, T);
    for (int e = threadIdx.x; e < n; e += RES_THREADS) lam[e] = make_float2(lam[e].x + phi[e].x, lam[e].y + phi[e].y);
    __syncthreads();
  }
  double acc = 0.0;
  for (int e = threadIdx.x; e < n; e += RES_THREADS)
    acc += (double)psi[e].x * (double)lam[e].x + (double)psi[e].y * (double)lam[e].y;
  *energy = H->constant + res_block_sum(acc, T);
  for (int j = J.n_reps + 1; j >= 1; --j) {
    if (res_cancelled(S, flag)) return FFGB_ERR_CANCELLED;
    const ResRot& vi = J.rot_inv[j - 1];
    res_rotate(psi, norb, na, nb, da, db, T.offa, T.offb, vi);
    res_phase(psi, norb, da, db, nullptr, vi.ang, T);
    res_rotate(lam, norb, na, nb, da, db, T.offa, T.offb, vi);
    res_phase(lam, norb, da, db, nullptr, vi.ang, T);
    res_trdm1(lam, psi, norb, da, db, T, S->dens[j - 1]);
    if (j > 1) {
      res_pair(lam, psi, norb, da, db, T, reinterpret_cast<double2*>(phi), S->dens[j - 1]);
      res_phase(psi, norb, da, db, &J.diag[j - 2], nullptr, T, -1.0);
      res_phase(lam, norb, da, db, &J.diag[j - 2], nullptr, T, -1.0);
    }
    __syncthreads();
  }
  return FFGB_OK;
}

__global__ void __launch_bounds__(RES_THREADS) resident_kernel(ResQueue* q, ResSlot* slots, int n_slots, ResDev* d,
                                                               unsigned long long idle_ns) {
  extern __shared__ __align__(16) unsigned char res_smem[];
  ResJob& J = *reinterpret_cast<ResJob*>(res_smem);
  float2* psi = reinterpret_cast<float2*>(res_smem + sizeof(ResJob));
  float2* phi = psi + RES_MAXDIM * RES_MAXDIM;
  __shared__ ResTables T;
  __shared__ long long s_ticket;
  __shared__ int s_flag;
  if (threadIdx.x == 0) atomicAdd(&d->running, 1);
  int exit_status = FFGB_OK;
  for (;;) {
    if (threadIdx.x == 0) s_ticket = res_claim(q, d, idle_ns);
    __syncthreads();
    const long long ticket = s_ticket;
    __syncthreads();
    if (ticket < 0) {
      exit_status = ticket == -1 ? FFGB_OK : FFGB_ERR_TIMEOUT;
      break;
    }
    ResSlot* S = slots + ticket % n_slots;
    {
      const int4* src = reinterpret_cast<const int4*>(&S->job);
      int4* dst = reinterpret_cast<int4*>(&J);
      for (int i = threadIdx.x; i < (int)(sizeof(ResJob) / 16); i += RES_THREADS) dst[i] = __ldcv(src + i);
    }
    if (threadIdx.x == 0) {
      // strings of both sectors in ascending integer (colex) order, and their indices
      int ka = 0, kb = 0;
      for (unsigned s = 0; s < 256u; ++s) T.ra[s] = T.rb[s] = -1;
      for (unsigned s = 0; s < (1u << J.norb); ++s) {
        const int pc = __popc(s);
        if (pc == J.na) {
          T.ra[s] = (short)ka;
          T.sa[ka++] = s;
        }
        if (pc == J.nb) {
          T.rb[s] = (short)kb;
          T.sb[kb++] = s;
        }
      }
    }
    __syncthreads();
    const int norb = J.norb, na = J.na, nb = J.nb;
    int da = 0, db = 0;
    for (unsigned s = 0; s < (1u << norb); ++s) {
      da += __popc(s) == na;
      db += __popc(s) == nb;
    }
    for (int j = threadIdx.x; j < RES_MAXDIM; j += RES_THREADS) {
      T.offa[j] = j * db;
      T.offb[j] = j;
    }
    const int n = da * db;
    for (int e = threadIdx.x; e < n; e += RES_THREADS) psi[e] = make_float2(e == 0 ? 1.f : 0.f, 0.f);
    __syncthreads();
    int status = FFGB_OK;
    double energy = 0.0;
    for (int k = 0; k <= J.n_reps && status == FFGB_OK; ++k) {
      if (res_cancelled(S, &s_flag)) {
        status = FFGB_ERR_CANCELLED;
        break;
      }
      res_rotate(psi, norb, na, nb, da, db, T.offa, T.offb, J.rot[k]);
      res_phase(psi, norb, da, db, k < J.n_reps ? &J.diag[k] : nullptr, J.rot[k].ang, T);
    }
    if (status == FFGB_OK && J.grad) {
      status = res_gradient(J, S, psi, phi, d->lam + (long long)blockIdx.x * RES_MAXDIM * RES_MAXDIM, da, db, T,
                            &s_flag, &energy);
    } else if (status == FFGB_OK) {
      const ResHam* H = J.ham;
      for (int t = 0; t < H->n_terms; ++t) {
        if ((t & 3) == 0 && res_cancelled(S, &s_flag)) {
          status = FFGB_ERR_CANCELLED;
          break;
        }
        {
          const float* src = reinterpret_cast<const float*>(H->rot + t);
          float* dst = reinterpret_cast<float*>(&T.trot);
          for (int i = threadIdx.x; i < (int)(sizeof(ResRot) / 4); i += RES_THREADS) dst[i] = src[i];
        }
        for (int e = threadIdx.x; e < n; e += RES_THREADS) phi[e] = psi[e];
        __syncthreads();
        res_rotate(phi, norb, na, nb, da, db, T.offa, T.offb, T.trot);
        energy += res_expect(phi, norb, da, db, H->z[t], T);
      }
      energy += H->constant;
    }
    __threadfence_system();  // this thread's density entries before the slot is marked done
    __syncthreads();
    if (threadIdx.x == 0) {
      S->energy = energy;
      S->status = status;
      st_release_sys(&S->state, RES_DONE);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicSub(&d->running, 1) == 1) {
      q->kstatus = exit_status;
      __threadfence_system();
    }
  }
}

constexpr size_t res_smem_bytes() { return sizeof(ResJob) + 2 * RES_MAXDIM * RES_MAXDIM * sizeof(float2); }

// --- host helpers -------------------------------------------------------------
using Mat = std::vector<cd>;

Mat res_load(const double* m, int n) {
  Mat a((size_t)n * n);
  for (int i = 0; i < n * n; ++i) a[i] = cd(m[2 * i], m[2 * i + 1]);
  return a;
}
Mat res_mul(const Mat& a, const Mat& b, int n) {
  Mat c((size_t)n * n, cd(0.0));
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j) c[i * n + j] += a[i * n + k] * b[k * n + j];
  return c;
}
Mat res_dag(const Mat& a, int n) {
  Mat c((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) c[i * n + j] = std::conj(a[j * n + i]);
  return c;
}
Mat res_eye(int n) {
  Mat c((size_t)n * n, cd(0.0));
  for (int i = 0; i < n; ++i) c[i * n + i] = 1.0;
  return c;
}

int res_plan(int norb, const Mat& V, ResRot& R) {
  std::memset(&R, 0, sizeof(R));
  if (norb == 0) return FFGB_OK;
  SectorPlan p;
  if (!plan_sector(norb, V.data(), true, p)) return fail(FFGB_ERR_NUMERIC, "orbital rotation plan failed");
  if (p.max_err > 1e-9) return fail(FFGB_ERR_NUMERIC, "orbital rotation is not unitary");
  if (p.kind != PLAN_FULL || (int)p.tri.size() != norb * (norb - 1) / 2)
    return fail(FFGB_ERR_UNSUPPORTED, "no brick network for this orbital rotation");
  for (size_t g = 0; g < p.tri.size(); ++g) {
    const double v[3] = {p.tri[g].c, p.tri[g].s.real(), p.tri[g].s.imag()};
    for (int q = 0; q < 3; ++q) {
      R.gp[3 * g + q] = (float)v[q];
      R.gl[3 * g + q] = (float)(v[q] - (double)(float)v[q]);
    }
  }
  for (int i = 0; i < norb; ++i) R.ang[i] = std::arg(p.diag[i]);
  return FFGB_OK;
}

// Diagonal Coulomb operator sum J^{st}_ij n_is n_jt / 2 (number rep.) or its
// Z-representation form, as in diag_coulomb_spec: same-spin diagonals halved
// (number rep.) or dropped (Z rep., with the 1/4 factor).
void res_coulomb(int norb, const double* aa, const double* ab, const double* bb, int zrep, ResDiag& D) {
  std::memset(&D, 0, sizeof(D));
  D.zrep = zrep;
  const double f = zrep ? 0.25 : 1.0;
  for (int i = 0; i < norb; ++i)
    for (int j = i; j < norb; ++j) {
      const double w = i == j ? (zrep ? 0.0 : 0.5) : 1.0;
      D.A[i][j] = f * w * aa[i * norb + j];
      D.B[i][j] = f * w * bb[i * norb + j];
    }
  for (int i = 0; i < norb; ++i)
    for (int j = 0; j < norb; ++j) D.X[i][j] = f * ab[i * norb + j];
}

}  // namespace
}  // namespace ffgb

using namespace ffgb;

struct ffgb_resident {
  int device = 0;
  int n_slots = 0, n_ctas = 0;
  unsigned long long idle_ns = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  bool launched = false;
  ResQueue* q = nullptr;  // host-mapped
  ResQueue* q_dev = nullptr;
  ResSlot* slots = nullptr;  // host-mapped
  ResSlot* slots_dev = nullptr;
  ResDev* dev = nullptr;  // device
  float2* lam = nullptr;  // device: per CTA the gradient's lambda
  std::vector<void*> hams;  // device blocks of the registered Hamiltonians
  std::vector<int> ham_norb;
  std::mutex mu;
  unsigned long long head = 0;  // next ticket (host copy of q->head)
};

static int res_publish(ffgb_resident* r, int ham_id, ResJob& job, long long* ticket);

static bool res_kernel_running(ffgb_resident* r) {
  if (!r->launched) return false;
  return cudaEventQuery(r->done) == cudaErrorNotReady;
}

static int res_launch(ffgb_resident* r) {
  FFGB_CUDA(cudaSetDevice(r->device));
  FFGB_CUDA(cudaMemsetAsync(&r->dev->running, 0, sizeof(int), r->stream));
  resident_kernel<<<r->n_ctas, RES_THREADS, res_smem_bytes(), r->stream>>>(r->q_dev, r->slots_dev, r->n_slots,
                                                                           r->dev, r->idle_ns);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  FFGB_CUDA(cudaEventRecord(r->done, r->stream));
  r->launched = true;
  return FFGB_OK;
}

extern "C" {

int ffgb_resident_open(int n_slots, int n_ctas, double idle_seconds, ffgb_resident** out) {
  g_err.clear();
  if (!out) return fail(FFGB_ERR_ARG, "out must not be NULL");
  *out = nullptr;
  if (n_slots < 1 || n_slots > (1 << 16)) return fail(FFGB_ERR_ARG, "n_slots must be in [1, 65536]");
  if (n_ctas < 1 || n_ctas > 1024) return fail(FFGB_ERR_ARG, "n_ctas must be in [1, 1024]");
  if (!(idle_seconds > 0.0) || idle_seconds > 3600.0) return fail(FFGB_ERR_ARG, "idle_seconds must be in (0, 3600]");
  auto r = std::make_unique<ffgb_resident>();
  FFGB_CUDA(cudaGetDevice(&r->device));
  r->n_slots = n_slots;
  r->n_ctas = n_ctas;
  r->idle_ns = (unsigned long long)(idle_seconds * 1e9);
  static std::atomic<unsigned long long> attr_ready{0};
  const unsigned long long bit = 1ull << (r->device & 63);
  if (!(attr_ready.load() & bit)) {
    FFGB_CUDA(cudaFuncSetAttribute(resident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)res_smem_bytes()));
    attr_ready.fetch_or(bit);
  }
  FFGB_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
  FFGB_CUDA(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming));
  FFGB_CUDA(cudaHostAlloc((void**)&r->q, sizeof(ResQueue), cudaHostAllocMapped));
  FFGB_CUDA(cudaHostAlloc((void**)&r->slots, sizeof(ResSlot) * (size_t)n_slots, cudaHostAllocMapped));
  std::memset(r->q, 0, sizeof(ResQueue));
  std::memset(r->slots, 0, sizeof(ResSlot) * (size_t)n_slots);
  FFGB_CUDA(cudaHostGetDevicePointer((void**)&r->q_dev, r->q, 0));
  FFGB_CUDA(cudaHostGetDevicePointer((void**)&r->slots_dev, r->slots, 0));
  FFGB_CUDA(cudaMalloc((void**)&r->dev, sizeof(ResDev)));
  count_alloc();
  FFGB_CUDA(cudaMalloc((void**)&r->lam, sizeof(float2) * RES_MAXDIM * RES_MAXDIM * (size_t)n_ctas));
  count_alloc();
  {
    ResDev d0;
    std::memset(&d0, 0, sizeof(d0));
    d0.lam = r->lam;
    FFGB_CUDA(cudaMemcpy(r->dev, &d0, sizeof(d0), cudaMemcpyHostToDevice));
  }
  *out = r.release();
  return FFGB_OK;
}

int ffgb_resident_hamiltonian(ffgb_resident* r, int norb, const double* one_body, int n_terms, const double* dcm,
                              const double* rots, double constant, int zrep, int* ham_id) {
  g_err.clear();
  if (!r || !ham_id) return fail(FFGB_ERR_ARG, "NULL argument");
  if (norb < 1 || norb > RES_MAXN) return fail(FFGB_ERR_UNSUPPORTED, "the resident evaluator takes norb in [1, 8]");
  if (n_terms < 0 || n_terms + 1 > RES_MAX_TERMS) return fail(FFGB_ERR_ARG, "n_terms out of range");
  if (n_terms > 0 && (!dcm || !rots)) return fail(FFGB_ERR_ARG, "dcm and rots must not be NULL");
  std::vector<ResRot> R, RU;
  std::vector<ResDiag> Z;
  if (one_body) {
    const Mat K = res_load(one_body, norb);
    std::vector<double> w;
    Mat vecs;
    hermitian_eigh(norb, K.data(), w, vecs);
    ResRot rr, ru;
    FFGB_TRY(res_plan(norb, res_dag(vecs, norb), rr));
    FFGB_TRY(res_plan(norb, vecs, ru));
    RU.push_back(ru);
    ResDiag zz;
    std::memset(&zz, 0, sizeof(zz));
    for (int i = 0; i < norb; ++i) zz.A[i][i] = zz.B[i][i] = w[i];
    R.push_back(rr);
    Z.push_back(zz);
  }
  for (int t = 0; t < n_terms; ++t) {
    const Mat U = res_load(rots + (size_t)t * norb * norb * 2, norb);
    ResRot rr, ru;
    FFGB_TRY(res_plan(norb, res_dag(U, norb), rr));
    FFGB_TRY(res_plan(norb, U, ru));
    RU.push_back(ru);
    const double* J = dcm + (size_t)t * norb * norb;
    ResDiag zz;
    res_coulomb(norb, J, J, J, zrep, zz);
    R.push_back(rr);
    Z.push_back(zz);
  }
  const size_t nt = R.size();
  const size_t bytes = sizeof(ResHam) + 64 + nt * (2 * sizeof(ResRot) + sizeof(ResDiag));
  std::vector<unsigned char> host(bytes, 0);
  void* blk = nullptr;
  FFGB_CUDA(cudaSetDevice(r->device));
  FFGB_CUDA(cudaMalloc(&blk, bytes));
  count_alloc();
  const size_t off_rot = (sizeof(ResHam) + 63) / 64 * 64;
  const size_t off_ru = off_rot + nt * sizeof(ResRot);
  const size_t off_z = off_ru + nt * sizeof(ResRot);
  ResHam h;
  h.norb = norb;
  h.n_terms = (int)nt;
  h.constant = constant;
  h.rot = reinterpret_cast<const ResRot*>((unsigned char*)blk + off_rot);
  h.rot_u = reinterpret_cast<const ResRot*>((unsigned char*)blk + off_ru);
  h.z = reinterpret_cast<const ResDiag*>((unsigned char*)blk + off_z);
  std::memcpy(host.data(), &h, sizeof(h));
  if (nt) {
    std::memcpy(host.data() + off_rot, R.data(), nt * sizeof(ResRot));
    std::memcpy(host.data() + off_ru, RU.data(), nt * sizeof(ResRot));
    std::memcpy(host.data() + off_z, Z.data(), nt * sizeof(ResDiag));
  }
  const cudaError_t e = cudaMemcpy(blk, host.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(blk);
    return fail(FFGB_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  std::lock_guard<std::mutex> lk(r->mu);
  r->hams.push_back(blk);
  r->ham_norb.push_back(norb);
  *ham_id = (int)r->hams.size() - 1;
  return FFGB_OK;
}

int ffgb_resident_submit(ffgb_resident* r, int ham_id, int norb, int na, int nb, int n_reps, const double* ucj_dcm,
                         const double* ucj_rots, const double* ucj_final, long long* ticket) {
  g_err.clear();
  if (!r || !ticket) return fail(FFGB_ERR_ARG, "NULL argument");
  if (norb < 1 || norb > RES_MAXN) return fail(FFGB_ERR_UNSUPPORTED, "the resident evaluator takes norb in [1, 8]");
  if (na < 0 || na > norb || nb < 0 || nb > norb) return fail(FFGB_ERR_ARG, "invalid electron numbers");
  if (n_reps < 1 || n_reps > RES_MAX_REPS)
    return fail(FFGB_ERR_UNSUPPORTED, "the resident evaluator takes n_reps in [1, 4]");
  if (!ucj_dcm || !ucj_rots) return fail(FFGB_ERR_ARG, "ucj_dcm and ucj_rots must not be NULL");
  {
    std::lock_guard<std::mutex> lk(r->mu);
    if (ham_id < 0 || ham_id >= (int)r->hams.size()) return fail(FFGB_ERR_ARG, "unknown Hamiltonian");
    if (r->ham_norb[ham_id] != norb) return fail(FFGB_ERR_ARG, "the Hamiltonian acts on another number of orbitals");
  }
  // host side of the circuit: merged rotations and phase gates (FP64)
  auto job = std::make_unique<ResJob>();
  std::memset(job.get(), 0, sizeof(ResJob));
  job->norb = norb;
  job->na = na;
  job->nb = nb;
  job->n_reps = n_reps;
  Mat basis = res_eye(norb);
  for (int k = 0; k < n_reps; ++k) {
    const Mat U = res_load(ucj_rots + (size_t)k * norb * norb * 2, norb);
    FFGB_TRY(res_plan(norb, res_mul(res_dag(U, norb), basis, norb), job->rot[k]));
    const double* J = ucj_dcm + (size_t)k * 2 * norb * norb;
    res_coulomb(norb, J, J + norb * norb, J, 0, job->diag[k]);
    basis = U;
  }
  if (ucj_final) basis = res_mul(res_load(ucj_final, norb), basis, norb);
  FFGB_TRY(res_plan(norb, basis, job->rot[n_reps]));
  return res_publish(r, ham_id, *job, ticket);
}

int ffgb_resident_submit_grad(ffgb_resident* r, int ham_id, int norb, int na, int nb, int n_reps,
                              const double* rots, const double* ucj_dcm, long long* ticket) {
  g_err.clear();
  if (!r || !ticket) return fail(FFGB_ERR_ARG, "NULL argument");
  if (norb < 1 || norb > RES_MAXN) return fail(FFGB_ERR_UNSUPPORTED, "the resident evaluator takes norb in [1, 8]");
  if (na < 0 || na > norb || nb < 0 || nb > norb) return fail(FFGB_ERR_ARG, "invalid electron numbers");
  if (n_reps < 1 || n_reps > RES_MAX_REPS)
    return fail(FFGB_ERR_UNSUPPORTED, "the resident evaluator takes n_reps in [1, 4]");
  if (!ucj_dcm || !rots) return fail(FFGB_ERR_ARG, "ucj_dcm and rots must not be NULL");
  {
    std::lock_guard<std::mutex> lk(r->mu);
    if (ham_id < 0 || ham_id >= (int)r->hams.size()) return fail(FFGB_ERR_ARG, "unknown Hamiltonian");
    if (r->ham_norb[ham_id] != norb) return fail(FFGB_ERR_ARG, "the Hamiltonian acts on another number of orbitals");
  }
  auto job = std::make_unique<ResJob>();
  std::memset(job.get(), 0, sizeof(ResJob));
  job->norb = norb;
  job->na = na;
  job->nb = nb;
  job->n_reps = n_reps;
  job->grad = 1;
  for (int k = 0; k <= n_reps; ++k) {
    const Mat V = res_load(rots + (size_t)k * norb * norb * 2, norb);
    FFGB_TRY(res_plan(norb, V, job->rot[k]));
    FFGB_TRY(res_plan(norb, res_dag(V, norb), job->rot_inv[k]));
  }
  for (int k = 0; k < n_reps; ++k) {
    const double* J = ucj_dcm + (size_t)k * 2 * norb * norb;
    res_coulomb(norb, J, J + norb * norb, J, 0, job->diag[k]);
  }
  return res_publish(r, ham_id, *job, ticket);
}

int ffgb_resident_poll_densities(ffgb_resident* r, long long ticket, double* energy, double* dens) {
  g_err.clear();
  if (!r || !energy || !dens) return fail(FFGB_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(r->mu);
  if (ticket < 0 || (unsigned long long)ticket >= r->head || r->head - (unsigned long long)ticket > (unsigned)r->n_slots)
    return fail(FFGB_ERR_ARG, "unknown ticket");
  ResSlot& S = r->slots[(unsigned long long)ticket % (unsigned long long)r->n_slots];
  const int st = __atomic_load_n(&S.state, __ATOMIC_ACQUIRE);
  if (st == RES_FREE) return fail(FFGB_ERR_ARG, "ticket already collected");
  if (!S.job.grad) return fail(FFGB_ERR_ARG, "not a gradient request");
  if (st != RES_DONE) {
    if (!res_kernel_running(r)) FFGB_TRY(res_launch(r));
    return FFGB_PENDING;
  }
  const int status = S.status;
  *energy = S.energy;
  const int n = S.job.norb, L = S.job.n_reps;
  for (int j = 0; j <= L; ++j)
    for (int blk = 0; blk < RES_DENS_BLOCKS; ++blk)
      for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) {
          const double2 v = (j == 0 && blk >= 2) ? make_double2(0.0, 0.0) : S.dens[j][blk][p * RES_MAXN + q];
          const size_t o = 2 * ((((size_t)j * RES_DENS_BLOCKS + blk) * n + p) * n + q);
          dens[o] = v.x;
          dens[o + 1] = v.y;
        }
  __atomic_store_n(&S.state, RES_FREE, __ATOMIC_RELEASE);
  if (status == FFGB_ERR_CANCELLED) return fail(FFGB_ERR_CANCELLED, "request cancelled");
  if (status != FFGB_OK) return fail(status, "resident evaluation failed");
  return FFGB_OK;
}

}  // extern "C"

static int res_publish(ffgb_resident* r, int ham_id, ResJob& job_in, long long* ticket) {
  ResJob* job = &job_in;
  std::lock_guard<std::mutex> lk(r->mu);
  job->ham = reinterpret_cast<const ResHam*>(r->hams[ham_id]);
  const unsigned long long t = r->head;
  ResSlot& S = r->slots[t % (unsigned long long)r->n_slots];
  if (__atomic_load_n(&S.state, __ATOMIC_ACQUIRE) != RES_FREE)
    return fail(FFGB_ERR_OOM, "resident queue full (collect finished requests with ffgb_resident_poll)");
  std::memcpy(&S.job, job, sizeof(ResJob));
  S.cancel = 0;
  S.status = 0;
  S.energy = 0.0;
  __atomic_store_n(&S.state, RES_READY, __ATOMIC_RELEASE);
  r->head = t + 1;
  __atomic_store_n(&r->q->head, t + 1, __ATOMIC_RELEASE);
  if (!res_kernel_running(r)) FFGB_TRY(res_launch(r));
  *ticket = (long long)t;
  return FFGB_OK;
}

extern "C" {

int ffgb_resident_poll(ffgb_resident* r, long long ticket, double* energy) {
  g_err.clear();
  if (!r || !energy) return fail(FFGB_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(r->mu);
  if (ticket < 0 || (unsigned long long)ticket >= r->head || r->head - (unsigned long long)ticket > (unsigned)r->n_slots)
    return fail(FFGB_ERR_ARG, "unknown ticket");
  ResSlot& S = r->slots[(unsigned long long)ticket % (unsigned long long)r->n_slots];
  const int st = __atomic_load_n(&S.state, __ATOMIC_ACQUIRE);
  if (st == RES_FREE) return fail(FFGB_ERR_ARG, "ticket already collected");
  if (S.job.grad) return fail(FFGB_ERR_ARG, "a gradient request: collect it with ffgb_resident_poll_densities");
  if (st != RES_DONE) {
    // a job that is not done while no kernel runs has not been claimed: relaunch
    if (!res_kernel_running(r)) FFGB_TRY(res_launch(r));
    return FFGB_PENDING;
  }
  const int status = S.status;
  *energy = S.energy;
  __atomic_store_n(&S.state, RES_FREE, __ATOMIC_RELEASE);
  if (status == FFGB_ERR_CANCELLED) return fail(FFGB_ERR_CANCELLED, "request cancelled");
  if (status != FFGB_OK) return fail(status, "resident evaluation failed");
  return FFGB_OK;
}

int ffgb_resident_cancel(ffgb_resident* r, long long ticket) {
  g_err.clear();
  if (!r) return fail(FFGB_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(r->mu);
  if (ticket < 0 || (unsigned long long)ticket >= r->head || r->head - (unsigned long long)ticket > (unsigned)r->n_slots)
    return fail(FFGB_ERR_ARG, "unknown ticket");
  ResSlot& S = r->slots[(unsigned long long)ticket % (unsigned long long)r->n_slots];
  __atomic_store_n(&S.cancel, 1, __ATOMIC_RELEASE);
  return FFGB_OK;
}

int ffgb_resident_start(ffgb_resident* r) {
  g_err.clear();
  if (!r) return fail(FFGB_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(r->mu);
  if (!res_kernel_running(r)) FFGB_TRY(res_launch(r));
  return FFGB_OK;
}

int ffgb_resident_status(ffgb_resident* r, int* running, int* kernel_status) {
  g_err.clear();
  if (!r || !running || !kernel_status) return fail(FFGB_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(r->mu);
  *running = res_kernel_running(r) ? 1 : 0;
  *kernel_status = *running ? FFGB_OK : __atomic_load_n(&r->q->kstatus, __ATOMIC_ACQUIRE);
  if (r->launched && !*running) {
    const cudaError_t e = cudaEventQuery(r->done);
    if (e != cudaSuccess) return fail(FFGB_ERR_CUDA, std::string("resident kernel: ") + cudaGetErrorString(e));
  }
  return FFGB_OK;
}

int ffgb_resident_close(ffgb_resident* r) {
  g_err.clear();
  if (!r) return FFGB_OK;
  int rc = FFGB_OK;
  cudaSetDevice(r->device);
  if (r->q) __atomic_store_n(&r->q->stop, 1, __ATOMIC_RELEASE);
  if (r->stream && cudaStreamSynchronize(r->stream) != cudaSuccess)
    rc = fail(FFGB_ERR_CUDA, "resident kernel did not finish cleanly");
  for (void* h : r->hams) cudaFree(h);
  if (r->dev) cudaFree(r->dev);
  if (r->lam) cudaFree(r->lam);
  if (r->slots) cudaFreeHost(r->slots);
  if (r->q) cudaFreeHost(r->q);
  if (r->done) cudaEventDestroy(r->done);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
  return rc;
}

}  // extern "C"
