// Persistent batched CG on diagonal-structured systems: the whole solve of
// every system in a batch -- initial residual, iterations, periodic FP64
// residual refinement, verification, fallback -- in ONE cooperative launch.
//
// Follows tbsla::mpi::Matrix::CG (src/mpi/matrix/CG.cpp:32-73) restated as
// in kernels/cg.cu (q = A p, alpha = r.z / p.q, beta = r_new.z_new / r.z,
// relative stop test confirmed on the FP64 true residual b - A x).
//
// Layout (DIA): a system whose entries lie on at most 8 diagonals (col - row
// = delta, the same deltas on every row of the system: 7-point stencils have
// 0, +-1, +-n, +-n^2) stores its values slot-major, a[k * n + i] = the entry
// of row i on the system's k-th diagonal (0 where the row has none), with the
// deltas in a per-system table.  Every "gather" of a neighbour is then a
// shifted contiguous stream: coalesced, no column indices in memory.
//
// Precision: with FP32 / BF16 storage the iteration runs entirely in FP32
// (vectors and arithmetic; reductions summed in FP32 per warp and FP64
// across warps), as the inner solver of FP64 iterative refinement: every
// `refresh` iterations, and whenever the recursive residual says converged,
// x += d (the FP32 correction) in FP64, r = b - A64 x in FP64 from the FP64
// values, and the iteration restarts from that residual.  GB300's FP64 pipe
// retires about 2 multiply-adds per clock per SM against 128 in FP32, so
// FP64 only where it decides the answer.  FP64 storage runs the same loop in
// FP64 with no periodic refresh.
//
// Preconditioners, per system: 0 none, 1 Jacobi (z = D^-1 r, D^-1 in FP32),
// 2 factored z = L (L^T r) with L lower-triangular on at most 8 diagonals
// (stored in FP32 or BF16, applied in T arithmetic).  Mode 2 falls back to
// Jacobi for the system (fallback code in its status) when its factor holds
// a non-finite value or a diagonal entry <= 0 (checked before the first
// iteration), when a refinement cycle does not lower its FP64 true residual
// (or, over 25 iterations or more, cuts its norm by less than 10%), or when
// r.z stops being positive and finite.
//
// One iteration, all systems at once, grid-wide barriers between phases:
//   A   q = A p; p.q              (modes 0/1 form p = z + beta p_old on the
//                                   fly and write it)
//   B   modes 0/1: alpha; d += alpha p; r -= alpha q; z = M r; r.z, r.r
//   B'  mode 2: r -= alpha q, and t = L^T r_new formed from r_old and q at
//       the row's upper neighbours (so no extra pass), r.z = t.t, r.r
//   D   mode 2: d += alpha p (for the systems B' stopped too); z = L t,
//       p = z + beta p
// Jacobi costs two barriers per iteration, the factored form three.
//
// Per-system scalars are kept in shared memory by every CTA and updated
// redundantly from the same global sums after each barrier, so no CTA waits
// for another to publish them.  The sums rotate through three accumulator
// slots: CTA 0 clears the slot two phases ahead, which no CTA reads or
// writes at that time.
//
// Every grid-wide wait is bounded (`wait_ns`, globaltimer): a CTA whose wait
// runs out sets the error word and returns, and every other CTA returns at
// its next wait; the host then reports TBSLA_ERR_TIMEOUT.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.hpp"

namespace tbsla_gpu {

namespace {

constexpr int PNT = 256;  // threads per CTA
constexpr int KMAX = kDiaMaxDiag;

// local states of a system
enum { S_ACTIVE = 0, S_CHECK = 1, S_RESTART_F = 2, S_DONE = 3, S_STOPPED = 4 };

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class T, class V>
__device__ __forceinline__ T val(V v);
template <>
__device__ __forceinline__ float val<float, float>(float v) { return v; }
template <>
__device__ __forceinline__ float val<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ double val<double, double>(double v) { return v; }
template <>
__device__ __forceinline__ double val<double, float>(float v) { return widen(v); }
template <>
__device__ __forceinline__ double val<double, __nv_bfloat16>(__nv_bfloat16 v) { return widen(v); }

__device__ __forceinline__ bool finite_v(float v) { return isfinite(v); }
__device__ __forceinline__ bool finite_v(__nv_bfloat16 v) { return isfinite(__bfloat162float(v)); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier with a bounded wait.  bar[0] arrival count, bar[1]
// generation, bar[2] error word.  Returns false when the grid must stop.
__device__ bool grid_sync(unsigned* bar, unsigned& gen, long long wait_ns, int* s_stop) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = gen + 1;
    __threadfence();
    const unsigned arrived = atomicAdd(&bar[0], 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicExch(&bar[1], target);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire(&bar[1]) != target) {
        if (ld_acquire(&bar[2]) != 0u) break;
        if ((long long)(global_ns() - t0) > wait_ns) {
          atomicExch(&bar[2], 1u);
          break;
        }
        __nanosleep(32);
      }
    }
    gen = target;
    __threadfence();
    *s_stop = ld_acquire(&bar[2]) != 0u;
  }
  __syncthreads();
  return !*s_stop;
}

// ---- 4-row vectors (FP32 iteration) --------------------------------------------
// With every system's first row and size a multiple of 4, a thread takes 4
// consecutive rows: own-row streams are 16-byte loads, and the rows of a
// neighbour diagonal, [i0 + s, i0 + s + 4), are put together from the two
// aligned vectors that cover them.  An aligned vector lies wholly inside or
// wholly outside its system, so rows outside read as 0 (their slot value is
// 0 too).  Every row's arithmetic is that of the scalar loops.
__device__ __forceinline__ float4 f4zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 ld4(const __nv_bfloat16* p) {
  const uint2 u = *reinterpret_cast<const uint2*>(p);
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                     __uint_as_float(u.y & 0xffff0000u));
}
__device__ __forceinline__ float4 ld4_stream(const float* p, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float4 ld4_stream(const __nv_bfloat16* p, uint64_t pol) {
  unsigned a, b;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
               : "=r"(a), "=r"(b) : "l"(p), "l"(pol));
  return make_float4(__uint_as_float(a << 16), __uint_as_float(a & 0xffff0000u), __uint_as_float(b << 16),
                     __uint_as_float(b & 0xffff0000u));
}
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
// The same with the shift's alignment class r = s & 3 given: a constant in
// the seven-point form of the kernel (the classes of a 7-point stencil whose
// plane and line sizes are multiples of 4), so each window's loads and lane
// shuffle are known when the kernel is compiled.
template <class E>
__device__ __forceinline__ float4 rows4r(const E* v, long i0, long s, int r, long lo, long hi) {
  const long b = i0 + s - r;
  const float4 v0 = b >= lo && b < hi ? ld4(v + b) : f4zero();
  if (r == 0) return v0;
  const float4 v1 = b + 4 >= lo && b + 4 < hi ? ld4(v + b + 4) : f4zero();
  if (r == 1) return make_float4(v0.y, v0.z, v0.w, v1.x);
  if (r == 2) return make_float4(v0.z, v0.w, v1.x, v1.y);
  return make_float4(v0.w, v1.x, v1.y, v1.z);
}
// Slot classes of the seven-point form: A's deltas ascending (-n^2, -n, -1,
// 0, +1, +n, +n^2), L's deltas (0, -1, -n, -n^2) and their negations.
__host__ __device__ constexpr int cls_a(int k) { return k == 2 ? 3 : (k == 4 ? 1 : 0); }
__host__ __device__ constexpr int cls_l(int k) { return k == 1 ? 3 : 0; }
__host__ __device__ constexpr int cls_lt(int k) { return k == 1 ? 1 : 0; }

__device__ __forceinline__ float4 fma4(float4 a, float4 b, float4 c) {
  return make_float4(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z), fmaf(a.w, b.w, c.w));
}
__device__ __forceinline__ float4 fma4s(float a, float4 b, float4 c) {
  return make_float4(fmaf(a, b.x, c.x), fmaf(a, b.y, c.y), fmaf(a, b.z, c.z), fmaf(a, b.w, c.w));
}
__device__ __forceinline__ float dot4(float4 a, float4 b, float acc) {
  return fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, fmaf(a.x, b.x, acc))));
}

// Per-warp running sums of up to 3 values for one system at a time: lanes
// add their rows' terms; when the warp moves to another system (or the phase
// ends) the warp reduces them and lane 0 adds them to acc[what * ns + sys] in
// FP64.  No CTA-wide barrier.  Every lane of the warp calls to() / flush()
// at the same points (a unit belongs to one warp and one system).
template <class T, int NV>
struct WarpSums {
  int sys = -1;
  T v[NV];
  __device__ __forceinline__ WarpSums() {
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = (T)0;
  }
  __device__ __forceinline__ void flush(double* acc, int ns) {
    if (sys >= 0) {
#pragma unroll
      for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
      }
      if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) atomicAdd(acc + (size_t)k * ns + sys, (double)v[k]);
      }
#pragma unroll
      for (int k = 0; k < NV; k++) v[k] = (T)0;
    }
    sys = -1;
  }
  __device__ __forceinline__ void to(int s, double* acc, int ns) {
    if (s != sys) {
      flush(acc, ns);
      sys = s;
    }
  }
};

// A phase works on the rows of the systems it selects (SELECT: the systems
// in a given state); every CTA computes the same selection from its own copy
// of the states.  The rows are cut into warp units -- 32 threads x the rows
// per thread (128 rows with 4 per thread, 32 with 1), never across a system
// -- and the warps of the grid take the selected units grid-stride: at any
// moment the whole grid works on one compact window of rows, so each
// array is read as one front sweeping through memory (many streams at
// scattered places ran at about 45% of the HBM bandwidth, against 98% for
// the same loads swept grid-stride), and every warp gets an even share
// whatever systems have finished.
#define SELECT(cond)                        \
  select_sys([&](int s_) { return (cond); }); \
  const int nsel_ = s_nsel
// A warp keeps the system of its last unit and that system's range of
// selected units [uk0_, uk1_): its next unit (a grid's worth of units on)
// usually lies in the same system, and then needs no search.
#define FOR_CHUNKS(ch)                                                                          \
  for (int ku_ = blockIdx.x * (PNT / 32) + warp_, us_ = -1, uk0_ = 0, uk1_ = 0; ku_ < nsel_; \
       ku_ += gridDim.x * (PNT / 32))                                                           \
    for (int ch_sys = (ku_ >= uk0_ && ku_ < uk1_)                                               \
                          ? us_                                                                 \
                          : (us_ = unit_sys(ku_), uk1_ = s_end[us_],                            \
                             uk0_ = uk1_ - (s_su[us_ + 1] - s_su[us_]), us_),                   \
             ch_r0 = (int)(s_off[ch_sys] + (long)(ku_ - uk0_) * urows),                         \
             ch_r1 = (int)min((long)ch_r0 + urows, s_off[ch_sys + 1]), once_ = 1;              \
         once_; once_ = 0)

// Three CTAs per SM (80 registers): the phases are bound by the bytes each
// SM keeps in flight, and 24 warps per SM measured 8% faster than 16 (the
// 128-register form) on the 32 x 128^3 learned batch, 21% on the 64-system
// batch; 4 CTAs (64 registers) spill in the 4-row paths.
template <class T, class V, class LV, int ST7>
__global__ void __launch_bounds__(PNT, 3) k_cg_persistent(DiaCg c) {
  // ST7: every system is a 7-point stencil in the seven-point form (K = 7,
  // KL = 4, slot classes cls_a / cls_l), checked by the host
  const int KA = ST7 ? 7 : c.K, KF = ST7 ? 4 : c.KL;
  __shared__ double s_rz[kDiaMaxSys], s_alpha[kDiaMaxSys], s_beta[kDiaMaxSys], s_bb[kDiaMaxSys],
      s_prev[kDiaMaxSys], s_rzj[kDiaMaxSys];
  __shared__ int s_st[kDiaMaxSys], s_mode[kDiaMaxSys], s_it[kDiaMaxSys], s_since[kDiaMaxSys], s_fb[kDiaMaxSys];
  __shared__ int s_stop;
  __shared__ long s_off[kDiaMaxSys + 1];  // first row of each system
  __shared__ int s_su[kDiaMaxSys + 1];    // first warp unit of each system, then the unit count
  __shared__ int s_end[kDiaMaxSys];       // selected units of systems 0..s
  __shared__ int s_nsel;
  __shared__ int s_ad[kDiaMaxSys * KMAX], s_ld[kDiaMaxSys * KMAX];
  const int ns = c.nsys;
  const int tid = threadIdx.x;
  const int lane_ = tid & 31, warp_ = tid >> 5;
  const int urows = c.vec4 ? 128 : 32;  // rows of a warp unit
  const long n = c.n;
  const V* __restrict__ A = static_cast<const V*>(c.avals);
  const LV* __restrict__ Lv = static_cast<const LV*>(c.lvals);
  T* __restrict__ D = static_cast<T*>(c.d);
  T* const R0 = static_cast<T*>(c.r0);
  T* const R1 = static_cast<T*>(c.r1);
  T* const P0 = static_cast<T*>(c.p0);
  T* const P1 = static_cast<T*>(c.p1);
  // the buffer of parity k (selects, not an indexed array: no local memory)
  auto R = [&](int k) { return (k & 1) ? R1 : R0; };
  auto P = [&](int k) { return (k & 1) ? P1 : P0; };
  T* __restrict__ Q = static_cast<T*>(c.q);
  T* __restrict__ Z = static_cast<T*>(c.z);
  T* __restrict__ Tt = static_cast<T*>(c.t);
  const float* __restrict__ dinv = c.dinv;
  const uint64_t pol = policy_evict_first();

  for (int s = tid; s <= ns; s += PNT) s_off[s] = c.sys_off[s];
  for (int t = tid; t < ns * KMAX; t += PNT) {
    s_ad[t] = c.adelta[t];
    s_ld[t] = c.ldelta ? c.ldelta[t] : 0;
  }
  __syncthreads();
  if (tid == 0) {
    int u = 0;
    for (int s = 0; s < ns; s++) {
      s_su[s] = u;
      u += (int)((s_off[s + 1] - s_off[s] + urows - 1) / urows);
    }
    s_su[ns] = u;
  }
  for (int s = tid; s < ns; s += PNT) {
    s_st[s] = S_CHECK;
    s_mode[s] = c.mode[s];
    s_it[s] = 0;
    s_since[s] = 0;
    s_fb[s] = 0;
    s_rz[s] = s_alpha[s] = s_beta[s] = s_bb[s] = s_rzj[s] = 0;
    s_prev[s] = __longlong_as_double(0x7ff0000000000000ll);  // +inf
  }
  __syncthreads();

  unsigned gen = 0;
  int ph = 0;  // phases done: accumulator slot of the current phase = ph % 3
  int g = 0;   // iteration parity of the R / P buffers
  bool init = true;
  auto slot = [&](int p) { return c.acc + (size_t)(p % 3) * 4 * ns; };
  // CTA 0 clears the slot two phases ahead (read at the start of the
  // previous phase by every CTA, written next in the following phase)
  auto clear_ahead = [&]() {
    if (blockIdx.x == 0) {
      double* a = slot(ph + 1);
      for (int t = tid; t < 4 * ns; t += PNT) a[t] = 0.0;
    }
  };
  auto any_state = [&](int st, int mode) {
    int f = 0;
    for (int s = tid; s < ns; s += PNT) f |= s_st[s] == st && (mode < 0 || s_mode[s] == mode);
    return __syncthreads_or(f) != 0;
  };
  // s_end / s_nsel for the systems where pred(s) holds (warp 0: a scan over
  // the systems, up to 8 per lane)
  auto select_sys = [&](auto pred) {
    __syncthreads();
    if (tid < 32) {
      const int per = (ns + 31) / 32, a0 = tid * per, a1 = min(a0 + per, ns);
      int cnt = 0;
      for (int s = a0; s < a1; s++)
        if (pred(s)) cnt += s_su[s + 1] - s_su[s];
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (tid >= o) incl += v;
      }
      int e = incl - cnt;
      for (int s = a0; s < a1; s++) {
        if (pred(s)) e += s_su[s + 1] - s_su[s];
        s_end[s] = e;
      }
      if (tid == 31) s_nsel = incl;
    }
    __syncthreads();
  };
  // the system of the k-th selected unit: the first whose s_end exceeds k
  auto unit_sys = [&](int k) {
    int lo = 0, hi = ns - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (s_end[mid] > k) hi = mid;
      else lo = mid + 1;
    }
    return lo;
  };
  // the delta tables, copied to shared memory once (every unit reads its
  // system's row of one of them)
  auto load_deltas = [&](const int* tab, int s, int kk, int (&dd)[KMAX]) {
    const int* t = tab == c.adelta ? s_ad : s_ld;
#pragma unroll
    for (int k = 0; k < KMAX; k++) dd[k] = k < kk ? t[s * KMAX + k] : 0;
  };

  for (;;) {
    // ================= refinement: systems in S_CHECK ======================
    if (any_state(S_CHECK, -1)) {
      // R1: x += d (FP64), d = 0; at the start, check the factors
      clear_ahead();
      {
        SELECT(s_st[s_] == S_CHECK);
        double* acc = slot(ph);
        WarpSums<float, 1> bad;
        FOR_CHUNKS(ch) {
          const int s = ch_sys;
          if (s_st[s] != S_CHECK) continue;
          const int r0 = ch_r0, r1 = ch_r1;
          const bool chk = init && s_mode[s] == 2;
          if (chk) bad.to(s, acc, ns);
          for (int i = r0 + lane_; i < r1; i += 32) {
            const double xi = c.x[i] + (double)D[i];
            if (isfinite(xi)) c.x[i] = xi;  // a non-finite correction is dropped
            D[i] = (T)0;
            if (chk) {
              for (int k = 0; k < c.KL; k++) {
                const LV lv = Lv[(size_t)k * n + i];
                if (!finite_v(lv)) bad.v[0] = 1.f;
                if (k == 0 && !(to_f(lv) > 0.f)) bad.v[0] = 1.f;  // slot 0 is the diagonal
              }
            }
          }
        }
        bad.flush(acc, ns);
      }
      if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
      {
        const double* acc = slot(ph);
        for (int s = tid; s < ns; s += PNT)
          if (s_st[s] == S_CHECK && init && s_mode[s] == 2 && acc[s] > 0) {
            s_mode[s] = 1;
            s_fb[s] = kFallbackBadFactor;
          }
        ph++;
      }
      __syncthreads();
      // R2: r = b - A64 x in FP64 (true residual), r.r; b.b at the start; the
      // Jacobi (or identity) z and r.z for a restart; p_old = 0
      clear_ahead();
      {
        SELECT(s_st[s_] == S_CHECK);
        double* acc = slot(ph);
        T* __restrict__ Rn = R(g);
        T* __restrict__ Po = P(g);
        WarpSums<double, 3> part;
        FOR_CHUNKS(ch) {
          const int s = ch_sys;
          if (s_st[s] != S_CHECK) continue;
          part.to(s, acc, ns);
          const int r0 = ch_r0, r1 = ch_r1;
          const long lo = c.sys_off[s], hi = c.sys_off[s + 1];
          int dd[KMAX];
          load_deltas(c.adelta, s, c.K, dd);
          const bool ident = s_mode[s] == 0;
          for (int i = r0 + lane_; i < r1; i += 32) {
            double ax = 0;
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
              if (k < c.K) {
                long j = i + dd[k];
                j = j < lo ? lo : (j >= hi ? hi - 1 : j);
                ax = fma_rn(ld_stream(c.a64 + (size_t)k * n + i, pol), c.x[j], ax);
              }
            }
            const double bi = c.b[i];
            const double ri = bi - ax;
            part.v[0] = fma_rn(ri, ri, part.v[0]);
            part.v[1] = fma_rn(bi, bi, part.v[1]);
            const T rt = (T)ri;
            Rn[i] = rt;
            const T zi = ident ? rt : (T)dinv[i] * rt;
            Z[i] = zi;
            part.v[2] += (double)(rt * zi);
            Po[i] = (T)0;
          }
        }
        part.flush(acc, ns);
      }
      if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
      {
        const double* acc = slot(ph);
        for (int s = tid; s < ns; s += PNT) {
          if (s_st[s] != S_CHECK) continue;
          const double rrt = acc[s];
          if (init) s_bb[s] = acc[ns + s];
          const double bb = s_bb[s];
          if (blockIdx.x == 0) c.relres[s] = bb > 0 ? sqrt(rrt / bb) : sqrt(rrt);
          if (rrt <= c.tol2 * bb) {
            s_st[s] = S_DONE;
          } else if (s_it[s] >= c.max_it) {
            s_st[s] = S_STOPPED;
          } else {
            // the factored iteration is given up when a refinement cycle did
            // not lower the FP64 true residual (or gave NaN), or when a cycle
            // of 25 iterations or more cut its norm by less than 10%
            // (squared: to above 0.81 of the last): progress too slow to keep
            const double keep_below = s_since[s] >= 25 ? 0.81 * s_prev[s] : s_prev[s];
            if (s_mode[s] == 2 && !init && !(rrt < keep_below)) {
              s_mode[s] = 1;
              s_fb[s] = kFallbackStagnation;
            }
            s_prev[s] = rrt;
            s_rzj[s] = acc[2 * ns + s];
            s_beta[s] = 0;
            s_since[s] = 0;
            if (s_mode[s] == 2) {
              s_st[s] = S_RESTART_F;
            } else {
              s_rz[s] = s_rzj[s];
              s_st[s] = S_ACTIVE;
            }
          }
        }
        ph++;
        init = false;
      }
      __syncthreads();
      if (any_state(S_RESTART_F, -1)) {
        // R3: t = L^T r (T arithmetic), r.z = t.t
        clear_ahead();
        {
          SELECT(s_st[s_] == S_RESTART_F);
          double* acc = slot(ph);
          const T* __restrict__ Rc = R(g);
          WarpSums<T, 1> part;
          FOR_CHUNKS(ch) {
            const int s = ch_sys;
            if (s_st[s] != S_RESTART_F) continue;
            part.to(s, acc, ns);
            const int r0 = ch_r0, r1 = ch_r1;
            const long hi = c.sys_off[s + 1];
            int ld[KMAX];
            load_deltas(c.ldelta, s, c.KL, ld);
            for (int i = r0 + lane_; i < r1; i += 32) {
              T t = (T)0;
#pragma unroll
              for (int k = 0; k < KMAX; k++) {
                if (k < c.KL) {
                  const long j = (long)i - ld[k];  // L_{j,i} sits on row j = i - delta
                  if (j < hi) t += val<T, LV>(Lv[(size_t)k * n + j]) * Rc[j];
                }
              }
              Tt[i] = t;
              part.v[0] += t * t;
            }
          }
          part.flush(acc, ns);
        }
        if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
        {
          const double* acc = slot(ph);
          for (int s = tid; s < ns; s += PNT) {
            if (s_st[s] != S_RESTART_F) continue;
            const double rz = acc[s];
            if (!(rz > 0) || !isfinite(rz)) {  // unusable factor: Jacobi from here
              s_mode[s] = 1;
              s_fb[s] = kFallbackStagnation;
              s_rz[s] = s_rzj[s];
              s_st[s] = S_ACTIVE;
            } else {
              s_rz[s] = rz;
            }
          }
          ph++;
        }
        __syncthreads();
        // R4: p = L t
        clear_ahead();
        {
          SELECT(s_st[s_] == S_RESTART_F);
          T* __restrict__ Po = P(g);
          FOR_CHUNKS(ch) {
            const int s = ch_sys;
            if (s_st[s] != S_RESTART_F) continue;
            const int r0 = ch_r0, r1 = ch_r1;
            const long lo = c.sys_off[s];
            int ld[KMAX];
            load_deltas(c.ldelta, s, c.KL, ld);
            for (int i = r0 + lane_; i < r1; i += 32) {
              T z = (T)0;
#pragma unroll
              for (int k = 0; k < KMAX; k++) {
                if (k < c.KL) {
                  long j = (long)i + ld[k];
                  j = j < lo ? lo : j;
                  z += val<T, LV>(Lv[(size_t)k * n + i]) * Tt[j];
                }
              }
              Po[i] = z;
            }
          }
        }
        if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
        for (int s = tid; s < ns; s += PNT)
          if (s_st[s] == S_RESTART_F) s_st[s] = S_ACTIVE;
        ph++;
        __syncthreads();
      }
    }
    if (!any_state(S_ACTIVE, -1)) break;

    // ================= one iteration =======================================
    const T* __restrict__ Pold = P(g);
    T* __restrict__ Pnew = P(g + 1);
    // A: q = A p, p.q
    clear_ahead();
    {
      SELECT(s_st[s_] == S_ACTIVE);
      double* acc = slot(ph);
      WarpSums<T, 1> part;
      FOR_CHUNKS(ch) {
        const int s = ch_sys;
        if (s_st[s] != S_ACTIVE) continue;
        part.to(s, acc, ns);
        const int r0 = ch_r0, r1 = ch_r1;
        const long lo = c.sys_off[s], hi = c.sys_off[s + 1];
        const bool fact = s_mode[s] == 2;
        int dd[KMAX];
        load_deltas(c.adelta, s, c.K, dd);
        const T beta = (T)s_beta[s];
        if constexpr (sizeof(T) == 4) {
          if (c.vec4) {
            const float* Zf = reinterpret_cast<const float*>(Z);
            const float* Pf = reinterpret_cast<const float*>(Pold);
            for (long i0 = r0 + 4 * lane_; i0 < r1; i0 += 128) {
              float4 a[KMAX];
#pragma unroll
              for (int k = 0; k < KMAX; k++) a[k] = k < KA ? ld4_stream(A + (size_t)k * n + i0, pol) : f4zero();
              float4 q = f4zero(), pi;
              if (fact) {
#pragma unroll
                for (int k = 0; k < KMAX; k++) {
                  const int r = ST7 ? cls_a(k) : (int)(dd[k] & 3);
                  if (k < KA) q = fma4(a[k], rows4r(Pf, i0, dd[k], r, lo, hi), q);
                }
                pi = ld4(Pf + i0);
              } else {
#pragma unroll
                for (int k = 0; k < KMAX; k++) {
                  const int r = ST7 ? cls_a(k) : (int)(dd[k] & 3);
                  if (k < KA)
                    q = fma4(a[k], fma4s(beta, rows4r(Pf, i0, dd[k], r, lo, hi), rows4r(Zf, i0, dd[k], r, lo, hi)), q);
                }
                pi = fma4s(beta, ld4(Pf + i0), ld4(Zf + i0));
                st4(reinterpret_cast<float*>(Pnew) + i0, pi);
              }
              st4(reinterpret_cast<float*>(Q) + i0, q);
              part.v[0] = dot4(pi, q, part.v[0]);
            }
            continue;
          }
        }
        for (int i = r0 + lane_; i < r1; i += 32) {
          T a[KMAX];
#pragma unroll
          for (int k = 0; k < KMAX; k++) a[k] = k < c.K ? val<T, V>(ld_stream(A + (size_t)k * n + i, pol)) : (T)0;
          T q = (T)0, pi;
          if (fact) {
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
              if (k < c.K) {
                long j = i + dd[k];
                j = j < lo ? lo : (j >= hi ? hi - 1 : j);
                q += a[k] * Pold[j];
              }
            }
            pi = Pold[i];
          } else {
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
              if (k < c.K) {
                long j = i + dd[k];
                j = j < lo ? lo : (j >= hi ? hi - 1 : j);
                q += a[k] * (Z[j] + beta * Pold[j]);
              }
            }
            pi = Z[i] + beta * Pold[i];
            Pnew[i] = pi;
          }
          Q[i] = q;
          part.v[0] += pi * q;
        }
      }
      part.flush(acc, ns);
    }
    if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
    {
      const double* acc = slot(ph);
      for (int s = tid; s < ns; s += PNT) {
        if (s_st[s] != S_ACTIVE) continue;
        const double pq = acc[s];
        s_alpha[s] = pq != 0 && isfinite(pq) ? s_rz[s] / pq : 0.0;
      }
      ph++;
    }
    __syncthreads();
    // B / B': residual update, preconditioner, r.z and r.r
    clear_ahead();
    {
      double* acc = slot(ph);
      SELECT(s_st[s_] == S_ACTIVE);
      const T* __restrict__ Ro = R(g);
      T* __restrict__ Rn = R(g + 1);
      WarpSums<T, 2> part;
      FOR_CHUNKS(ch) {
        const int s = ch_sys;
        if (s_st[s] != S_ACTIVE) continue;
        part.to(s, acc, ns);
        const int r0 = ch_r0, r1 = ch_r1;
        const T alpha = (T)s_alpha[s];
        const int mode = s_mode[s];
        if constexpr (sizeof(T) == 4) {
          if (c.vec4) {
            const long lo = c.sys_off[s], hi = c.sys_off[s + 1];
            float* Df = reinterpret_cast<float*>(D);
            const float* Rof = reinterpret_cast<const float*>(Ro);
            const float* Qf = reinterpret_cast<const float*>(Q);
            float* Rnf = reinterpret_cast<float*>(Rn);
            if (mode == 2) {
              int ld[KMAX];
              load_deltas(c.ldelta, s, c.KL, ld);
              // (d += alpha p is left to phase D, which reads p anyway)
              for (long i0 = r0 + 4 * lane_; i0 < r1; i0 += 128) {
                // every load before the first store (the stores could alias
                // them as far as the compiler knows, so a store in between
                // would hold the later loads back a whole memory round trip)
                const float4 ri = fma4s(-alpha, ld4(Qf + i0), ld4(Rof + i0));
                float4 t = f4zero();
                if constexpr (ST7 != 0) {
                  // L's slots 0 (delta 0) and 1 (rows i0 + 1 .. i0 + 4): the
                  // new residual of the row itself is ri, and three of the
                  // four shifted rows are ri's; only row i0 + 4 is formed
                  // anew (the same operations as the general loop below)
                  t = fma4(ld4(Lv + i0), ri, t);
                  const long j = i0 + 4;
                  const float rn = j < hi ? fmaf(-alpha, Qf[j], Rof[j]) : 0.f;
                  t = fma4(rows4r(Lv + (size_t)n, i0, 1, 1, lo, hi), make_float4(ri.y, ri.z, ri.w, rn), t);
                }
#pragma unroll
                for (int k = ST7 ? 2 : 0; k < KMAX; k++) {
                  if (k < KF) {
                    const long sh = -(long)ld[k];  // L_{j,i} sits on row j = i - delta
                    const int r = ST7 ? cls_lt(k) : (int)(sh & 3);
                    const float4 rf = fma4s(-alpha, rows4r(Qf, i0, sh, r, lo, hi), rows4r(Rof, i0, sh, r, lo, hi));
                    t = fma4(rows4r(Lv + (size_t)k * n, i0, sh, r, lo, hi), rf, t);
                  }
                }
                st4(Rnf + i0, ri);
                st4(reinterpret_cast<float*>(Tt) + i0, t);
                part.v[1] = dot4(ri, ri, part.v[1]);
                part.v[0] = dot4(t, t, part.v[0]);
              }
            } else {
              for (long i0 = r0 + 4 * lane_; i0 < r1; i0 += 128) {
                const float4 pn = ld4(reinterpret_cast<const float*>(Pnew) + i0), dold = ld4(Df + i0);
                const float4 ri = fma4s(-alpha, ld4(Qf + i0), ld4(Rof + i0));
                float4 zi = ri;
                if (mode == 1) {  // loaded before the stores, as above
                  const float4 dv = ld4(dinv + i0);
                  zi = make_float4(dv.x * ri.x, dv.y * ri.y, dv.z * ri.z, dv.w * ri.w);
                }
                st4(Df + i0, fma4s(alpha, pn, dold));
                st4(Rnf + i0, ri);
                st4(reinterpret_cast<float*>(Z) + i0, zi);
                part.v[0] = dot4(ri, zi, part.v[0]);
                part.v[1] = dot4(ri, ri, part.v[1]);
              }
            }
            continue;
          }
        }
        if (mode == 2) {
          const long hi = c.sys_off[s + 1];
          int ld[KMAX];
          load_deltas(c.ldelta, s, c.KL, ld);
          for (int i = r0 + lane_; i < r1; i += 32) {
            const T ri = Ro[i] - alpha * Q[i];
            T t = (T)0;
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
              if (k < c.KL) {
                const long j = (long)i - ld[k];
                if (j < hi) t += val<T, LV>(Lv[(size_t)k * n + j]) * (Ro[j] - alpha * Q[j]);
              }
            }
            Rn[i] = ri;  // the stores after every load
            Tt[i] = t;
            part.v[1] += ri * ri;
            part.v[0] += t * t;
          }
        } else {
          for (int i = r0 + lane_; i < r1; i += 32) {
            const T pn = Pnew[i], dold = D[i];
            const T ri = Ro[i] - alpha * Q[i];
            const T zi = mode == 1 ? (T)dinv[i] * ri : ri;
            D[i] = dold + alpha * pn;  // the stores after every load
            Rn[i] = ri;
            Z[i] = zi;
            part.v[0] += ri * zi;
            part.v[1] += ri * ri;
          }
        }
      }
      part.flush(acc, ns);
    }
    if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
    {
      const double* acc = slot(ph);
      for (int s = tid; s < ns; s += PNT) {
        if (s_st[s] != S_ACTIVE) continue;
        s_it[s]++;
        s_since[s]++;
        const double rzn = acc[s], rr = acc[ns + s];
        s_beta[s] = s_rz[s] != 0 ? rzn / s_rz[s] : 0.0;
        s_rz[s] = rzn;
        if (rr <= c.tol2 * s_bb[s])
          s_st[s] = S_CHECK;  // apparently converged: verify on the FP64 residual
        else if (s_it[s] >= c.max_it)
          s_st[s] = S_CHECK;  // iteration limit: final refinement
        else if (c.refresh > 0 && s_since[s] >= c.refresh)
          s_st[s] = S_CHECK;  // periodic refinement
        else if (!(rzn > 0) || !isfinite(rzn) || !isfinite(rr))
          s_st[s] = S_CHECK;  // breakdown: refine (and fall back if it does not help)
      }
      ph++;
    }
    __syncthreads();
    // factored systems still iterating, or just stopped by phase B' (which
    // leaves their d += alpha p to this phase)
    int fact_ = 0;
    for (int s = tid; s < ns; s += PNT) fact_ |= s_mode[s] == 2 && (s_st[s] == S_ACTIVE || s_st[s] == S_CHECK);
    if (__syncthreads_or(fact_)) {
      // D: d += alpha p; z = L t, p = z + beta p (iterating systems)
      clear_ahead();
      SELECT(s_mode[s_] == 2 && (s_st[s_] == S_ACTIVE || s_st[s_] == S_CHECK));
      FOR_CHUNKS(ch) {
        const int s = ch_sys;
        const bool act = s_st[s] == S_ACTIVE;
        const int r0 = ch_r0, r1 = ch_r1;
        const long lo = c.sys_off[s];
        const T alpha = (T)s_alpha[s];
        const T beta = (T)s_beta[s];
        int ld[KMAX];
        load_deltas(c.ldelta, s, c.KL, ld);
        if constexpr (sizeof(T) == 4) {
          if (c.vec4) {
            const long hi = c.sys_off[s + 1];
            const float* Tf = reinterpret_cast<const float*>(Tt);
            float* Df = reinterpret_cast<float*>(D);
            for (long i0 = r0 + 4 * lane_; i0 < r1; i0 += 128) {
              const float4 po = ld4(reinterpret_cast<const float*>(Pold) + i0), dold = ld4(Df + i0);
              float4 z = f4zero();
              if (act) {
                if constexpr (ST7 != 0) {
                  // slot 0 (the rows themselves) and slot 1 (rows i0 - 1 ..
                  // i0 + 2) from the rows' own vector of t and the one entry
                  // before it
                  const float4 t0 = ld4(Tf + i0);
                  z = fma4(ld4(Lv + i0), t0, z);
                  const float tm = i0 - 4 >= lo ? Tf[i0 - 1] : 0.f;
                  z = fma4(ld4(Lv + (size_t)n + i0), make_float4(tm, t0.x, t0.y, t0.z), z);
                }
#pragma unroll
                for (int k = ST7 ? 2 : 0; k < KMAX; k++) {
                  const int r = ST7 ? cls_l(k) : (int)(ld[k] & 3);
                  if (k < KF) z = fma4(ld4(Lv + (size_t)k * n + i0), rows4r(Tf, i0, ld[k], r, lo, hi), z);
                }
              }
              st4(Df + i0, fma4s(alpha, po, dold));
              if (act) st4(reinterpret_cast<float*>(Pnew) + i0, fma4s(beta, po, z));
            }
            continue;
          }
        }
        for (int i = r0 + lane_; i < r1; i += 32) {
          const T po = Pold[i], dold = D[i];
          T z = (T)0;
          if (act) {
#pragma unroll
            for (int k = 0; k < KMAX; k++) {
              if (k < c.KL) {
                long j = (long)i + ld[k];
                j = j < lo ? lo : j;
                z += val<T, LV>(Lv[(size_t)k * n + i]) * Tt[j];
              }
            }
          }
          D[i] = dold + alpha * po;
          if (act) Pnew[i] = z + beta * po;
        }
      }
      if (!grid_sync(c.bar, gen, c.wait_ns, &s_stop)) return;
      ph++;
    }
    g++;
  }

  // results (CTA 0)
  if (blockIdx.x == 0) {
    for (int s = tid; s < ns; s += PNT) {
      c.status[s] = s_st[s] == S_DONE ? kDone : kStopped;
      c.iters[s] = s_it[s];
      c.mode[s] = s_mode[s];
      c.fallback[s] = s_fb[s];
    }
  }
}
#undef FOR_CHUNKS
#undef SELECT

// ---- layout builders ----------------------------------------------------------

// a64[k * n + i] = entry of row i on diagonal k of its system (zeroed first by
// the caller); one thread per row over the concatenated CSR arrays.
__global__ void k_dia_fill(const int* __restrict__ rowptr, const int* __restrict__ colidx,
                           const double* __restrict__ vals, const int* __restrict__ row_sys,
                           const int* __restrict__ delta, int K, long n, double* __restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int s = row_sys[i];
    for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
      const long d = (long)colidx[e] - i;
      for (int k = 0; k < K; k++)
        if (delta[s * KMAX + k] == d) {
          out[(size_t)k * n + i] = vals[e];
          break;
        }
    }
  }
}

// 1 / a_ii in FP32 (1 where the diagonal is missing or zero).
__global__ void k_dia_dinv(const double* __restrict__ a64, const int* __restrict__ row_sys,
                           const int* __restrict__ delta, int K, long n, float* __restrict__ dinv) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int s = row_sys[i];
    double d = 0;
    for (int k = 0; k < K; k++)
      if (delta[s * KMAX + k] == 0) {  // the first slot of delta 0 (padding slots repeat it, zero-valued)
        d = a64[(size_t)k * n + i];
        break;
      }
    dinv[i] = d != 0 ? (float)(1.0 / d) : 1.f;
  }
}

template <class T, class V, class LV>
const void* kernel_of(bool st7) {
  if constexpr (sizeof(T) == 4) {
    if (st7) return (const void*)k_cg_persistent<T, V, LV, 1>;
  }
  return (const void*)k_cg_persistent<T, V, LV, 0>;
}

template <class T, class V, class LV>
cudaError_t launch_persistent(const DiaCg& c, int grid, cudaStream_t s) {
  void* args[] = {const_cast<DiaCg*>(&c)};
  return cudaLaunchCooperativeKernel(kernel_of<T, V, LV>(c.st7 != 0), dim3(grid), dim3(PNT), args, 0, s);
}

template <class T, class V, class LV>
int resident_grid(bool st7) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel_of<T, V, LV>(st7), PNT, 0) != cudaSuccess)
    return 0;
  return sms * per;
}

int variant(int prec, int lprec) {
  const int l = lprec == kBF16 ? 1 : 0;  // factor values: bfloat16 or float
  if (prec == kF64) return 0 + l;
  if (prec == kF32) return 2 + l;
  return 4 + l;
}

}  // namespace

int cg_dia_grid(int prec, int lprec, int st7) {
  switch (variant(prec, lprec)) {
    case 0: return resident_grid<double, double, float>(false);
    case 1: return resident_grid<double, double, __nv_bfloat16>(false);
    case 2: return resident_grid<float, float, float>(st7 != 0);
    case 3: return resident_grid<float, float, __nv_bfloat16>(st7 != 0);
    case 4: return resident_grid<float, __nv_bfloat16, float>(st7 != 0);
    case 5: return resident_grid<float, __nv_bfloat16, __nv_bfloat16>(st7 != 0);
  }
  return 0;
}

bool dia_seven_point(const int* adelta, const int* ldelta, int nsys, int K, int KL) {
  if (K != 7 || (ldelta && KL != 4)) return false;
  for (int s = 0; s < nsys; s++) {
    for (int k = 0; k < 7; k++)
      if ((adelta[s * kDiaMaxDiag + k] & 3) != cls_a(k)) return false;
    if (ldelta) {
      const int* l = ldelta + s * kDiaMaxDiag;
      for (int k = 0; k < 4; k++)
        if ((l[k] & 3) != cls_l(k)) return false;
      // phases B' and D take L's slots 0 and 1 from the rows' own vectors:
      // those two deltas must be exactly 0 and -1, not only of their class
      if (l[0] != 0 || l[1] != -1) return false;
    }
  }
  return true;
}

cudaError_t cg_dia_solve(const DiaCg& c, int grid, cudaStream_t s) {
  switch (variant(c.prec, c.lprec)) {
    case 0: return launch_persistent<double, double, float>(c, grid, s);
    case 1: return launch_persistent<double, double, __nv_bfloat16>(c, grid, s);
    case 2: return launch_persistent<float, float, float>(c, grid, s);
    case 3: return launch_persistent<float, float, __nv_bfloat16>(c, grid, s);
    case 4: return launch_persistent<float, __nv_bfloat16, float>(c, grid, s);
    case 5: return launch_persistent<float, __nv_bfloat16, __nv_bfloat16>(c, grid, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t dia_fill(const int* rowptr, const int* colidx, const double* vals, const int* row_sys,
                     const int* delta, int K, long n, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (int)std::min<long>((n + 255) / 256, 152L * 16);
  k_dia_fill<<<grid, 256, 0, s>>>(rowptr, colidx, vals, row_sys, delta, K, n, out);
  return cudaGetLastError();
}

cudaError_t dia_dinv(const double* a64, const int* row_sys, const int* delta, int K, long n, float* dinv,
                     cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (int)std::min<long>((n + 255) / 256, 152L * 16);
  k_dia_dinv<<<grid, 256, 0, s>>>(a64, row_sys, delta, K, n, dinv);
  return cudaGetLastError();
}

}  // namespace tbsla_gpu
