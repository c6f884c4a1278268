// Device code shared by the single-solve engine (hm2d.cu) and the batched
// ragged engine (batch.cu): the contact, wall, bond and indenter laws, the
// per-particle evaluation, the single-solve step kernels and the cell-list
// rebuild kernels. Kernels that the batched engine also runs take a MULTI
// flag: per-instance parameters, instance-local cell keys and live counts
// read from the control block.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "bulk.cuh"
#include "common.h"
#include "hm2d.cuh"
#include "tdem.h"

namespace tdem {
namespace hm {
// kBatch commits like kStep, except that an instance's first evaluation
// (primed == 0) applies the priming half kick of kPrime.
enum Mode { kPrime = 0, kStep = 1, kPeek = 2, kBatch = 3 };

template <class T>
__device__ __forceinline__ T dev_sqrt(T x);
template <>
__device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }
template <>
__device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }

template <class T>
struct PairOut {
  T fx, fy;   // force on a
  T cr;       // n x F_a (torque per unit lever)
  V2<T> xi;   // updated history (owner orientation)
  T diss;     // dissipated energy this step
  T un, ut;   // elastic energies (for the ledger read-back)
  bool active;
};

// Pair geometry from canonically ordered operands (a = lower sorted index):
// b - a through the integer cell difference plus the offset difference.
template <class T>
struct Geo {
  T dx, dy, d2, rs;
};

template <class T>
__device__ __forceinline__ Geo<T> pair_geo(const Params<T>& P, const V4<T>& a, const V4<T>& b) {
  const int ca = lane_to_cell(a.w), cb = lane_to_cell(b.w);
  Geo<T> g;
  g.dx = fma((T)((cb & 0xFFFF) - (ca & 0xFFFF)), P.cell, b.x - a.x);
  g.dy = fma((T)((cb >> 16) - (ca >> 16)), P.cell, b.y - a.y);
  g.d2 = g.dx * g.dx + g.dy * g.dy;
  g.rs = a.z + b.z;
  return g;
}

// Effective radius r_a r_b / (r_a + r_b) and effective mass 1 / (1/m_a + 1/m_b).
// FP32: reciprocals instead of divides (rcp_rn then a product: <= 1 ulp);
// _rn products are never fused, so every kernel computes the same bits.
template <class T>
__device__ __forceinline__ void pair_effective(T ra, T rb, T inv_ma, T inv_mb, T& reff, T& meff) {
  if constexpr (sizeof(T) == 4) {
    reff = __fmul_rn(__fmul_rn(ra, rb), __frcp_rn(ra + rb));
    meff = __frcp_rn(inv_ma + inv_mb);
  } else {
    reff = ra * rb / (ra + rb);
    meff = T(1) / (inv_ma + inv_mb);
  }
}

template <class T>
__device__ __forceinline__ PairOut<T> contact_law(const Params<T>& P, T delta, T nx, T ny, T reff, T meff, T ra,
                                                  T rb, const V4<T>& va, const V4<T>& vb, V2<T> xi);

// One active contact (g.d2 < g.rs^2): force on a, torque lever term, history.
template <class T>
__device__ __forceinline__ PairOut<T> pair_force(const Params<T>& P, const Geo<T>& g, const V4<T>& pa,
                                                 const V4<T>& va, const V4<T>& pb, const V4<T>& vb,
                                                 V2<T> xi) {
  if (!(va.w + vb.w > T(0))) {  // two clamped discs exchange no force
    PairOut<T> o;
    o.active = true;
    o.fx = o.fy = o.cr = o.diss = o.un = o.ut = T(0);
    o.xi = V2<T>{T(0), T(0)};
    return o;
  }
  const T d = dev_sqrt(g.d2);  // IEEE: the overlap rs - d is a small difference
  const T delta = g.rs - d;
  T nx, ny, reff, meff;
  if constexpr (sizeof(T) == 4) {
    const T inv_d = __frcp_rn(d);
    nx = __fmul_rn(g.dx, inv_d);
    ny = __fmul_rn(g.dy, inv_d);
  } else {
    nx = g.dx / d;
    ny = g.dy / d;
  }
  pair_effective<T>(pa.z, pb.z, va.w, vb.w, reff, meff);
  return contact_law<T>(P, delta, nx, ny, reff, meff, pa.z, pb.z, va, vb, xi);
}

// The contact law proper, from the overlap delta > 0 and the unit normal n
// from a to b: Hertz normal force with the Tsuji dashpot, clamped at zero;
// the tangential history incremented by the tangential relative velocity of
// the contact points and rotated into the current tangent plane; the Mindlin
// spring S_t xi capped at mu F_n with the state projected onto the cone.
template <class T>
__device__ __forceinline__ PairOut<T> contact_law(const Params<T>& P, T delta, T nx, T ny, T reff, T meff, T ra,
                                                  T rb, const V4<T>& va, const V4<T>& vb, V2<T> xi) {
  PairOut<T> o;
  o.active = true;
  const T sq = dev_sqrt(reff * delta);
  const T sn = P.estar2 * sq;
  const T fel = (T(2) / T(3)) * sn * delta;
  const T wsum = va.z * ra + vb.z * rb;
  const T vrx = (va.x - vb.x) - wsum * ny;
  const T vry = (va.y - vb.y) + wsum * nx;
  const T vn = vrx * nx + vry * ny;
  const T fn = fmax(fel + P.damp * dev_sqrt(sn * meff) * vn, T(0));
  const T vtx = vrx - vn * nx, vty = vry - vn * ny;
  T xx = xi.x + vtx * P.dt, xy = xi.y + vty * P.dt;
  const T xn = xx * nx + xy * ny;
  xx -= xn * nx;
  xy -= xn * ny;
  const T st = P.gstar8 * sq;
  const T fmag = st * dev_sqrt(xx * xx + xy * xy);
  const T cap = P.mu * fn;
  T diss = (fn - fel) * vn * P.dt;
  if (fmag > cap) {
    const T sc = cap / fmag;
    diss += cap * (fmag - cap) / st;
    xx *= sc;
    xy *= sc;
  }
  o.fx = -fn * nx - st * xx;
  o.fy = -fn * ny - st * xy;
  o.cr = nx * o.fy - ny * o.fx;
  o.xi.x = xx;
  o.xi.y = xy;
  o.diss = diss;
  o.un = T(0.4) * fel * delta;
  o.ut = T(0.5) * st * (xx * xx + xy * xy);
  return o;
}

// Planar wall with inward normal (nwx, nwy) at distance `gap` from the centre.
template <class T, bool COMMIT, class A>
__device__ __forceinline__ void wall_contact(const Params<T>& P, T nwx, T nwy, T gap, const V4<T>& p,
                                             const V4<T>& v, V2<T>* slot, A& fx, A& fy,
                                             A& tq, T& diss, T& un, T& ut, bool peek_old_xi) {
  V2<T> xw = *slot;
  const T delta = p.z - gap;
  if (!(delta > T(0))) {
    if (COMMIT && (xw.x != T(0) || xw.y != T(0))) *slot = V2<T>{T(0), T(0)};
    return;
  }
  const T r = p.z;
  const T m = T(1) / v.w;
  const T sq = dev_sqrt(r * delta);
  const T sn = P.estar2 * sq;
  const T fel = (T(2) / T(3)) * sn * delta;
  // contact point velocity v + omega x (-r n_w)
  const T vcx = v.x + v.z * r * nwy;
  const T vcy = v.y - v.z * r * nwx;
  const T vdot = vcx * nwx + vcy * nwy;
  const T vn = -vdot;
  const T fn = fmax(fel + P.damp * dev_sqrt(sn * m) * vn, T(0));
  const T vtx = vcx - vdot * nwx, vty = vcy - vdot * nwy;
  T xx = xw.x + vtx * P.dt, xy = xw.y + vty * P.dt;
  const T xn = xx * nwx + xy * nwy;
  xx -= xn * nwx;
  xy -= xn * nwy;
  const T st = P.gstar8 * sq;
  const T fmag = st * dev_sqrt(xx * xx + xy * xy);
  const T cap = P.mu_wall * fn;
  T d = (fn - fel) * vn * P.dt;
  if (fmag > cap) {
    const T s = cap / fmag;
    d += cap * (fmag - cap) / st;
    xx *= s;
    xy *= s;
  }
  const T f_x = fn * nwx - st * xx;
  const T f_y = fn * nwy - st * xy;
  fx.add(f_x);
  fy.add(f_y);
  tq.add(-r * (nwx * f_y - nwy * f_x));
  diss += d;
  un += T(0.4) * fel * delta;
  const T ux = peek_old_xi ? xw.x : xx, uy = peek_old_xi ? xw.y : xy;
  ut += T(0.5) * st * (ux * ux + uy * uy);
  if (COMMIT) *slot = V2<T>{xx, xy};
}

__device__ __forceinline__ double block_sum_d(double x) {
  __shared__ double s[kThreads / 32];
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = x;
  __syncthreads();
  double m = s[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m += s[w];
  __syncthreads();
  return m;
}

// Block sum of a per-thread value of the engine's type: the warp stage runs in
// T (GB300 executes FP64 at a small fraction of the FP32 rate), the eight warp
// totals are combined in double in warp order.
template <class T>
__device__ __forceinline__ double block_sum_t(T x) {
  __shared__ double s[kThreads / 32];
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = (double)x;
  __syncthreads();
  double m = s[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m += s[w];
  __syncthreads();
  return m;
}

// ---------------------------------------------------------------------------
// The step kernel: one thread per particle. MODE kPrime / kStep commit the
// evaluation (history, integrated state, ledger); kPeek only reports the
// integer-time velocity, force and energies.
// ---------------------------------------------------------------------------
// Where a particle reads its partners' state. GlobalFetch: the current
// buffers in HBM (through L2). WindowFetch: a shared-memory copy of a window
// of sorted indices [lo, hi) when the partner lies in it, else HBM; the copy
// holds the same values, so results are bit-identical either way.
template <class T>
struct GlobalFetch {
  const V4<T>* __restrict__ pos;
  const V4<T>* __restrict__ vel;
  __device__ __forceinline__ V4<T> p(int j) const { return pos[j]; }
  __device__ __forceinline__ V4<T> v(int j) const { return vel[j]; }
};

template <class T>
struct WindowFetch {
  const V4<T>* __restrict__ pos;   // HBM
  const V4<T>* __restrict__ vel;
  const V4<T>* spos;               // shared-memory rings: index j sits at (j - off) & mask
  const V4<T>* svel;
  int lo, hi, off, mask;
  __device__ __forceinline__ bool in(int j) const { return (unsigned)(j - lo) < (unsigned)(hi - lo); }
  __device__ __forceinline__ V4<T> p(int j) const { return in(j) ? spos[(j - off) & mask] : pos[j]; }
  __device__ __forceinline__ V4<T> v(int j) const { return in(j) ? svel[(j - off) & mask] : vel[j]; }
};

// One candidate slot of particle i (partner j at position q): contact test,
// history update in place, force and torque accumulation.
template <class T, int MODE, class F, class A>
__device__ __forceinline__ void do_slot(const Params<T>& P, const F& fetch,
                                        V2<T>* __restrict__ hist, int i, int j, int s, size_t slot,
                                        const V4<T>& p, const V4<T>& v, const V4<T>& q, unsigned mask,
                                        unsigned& nmask, A& fx, A& fy, A& tq, T& diss, T& un,
                                        T& ut, int primed) {
  constexpr bool COMMIT = MODE != kPeek;
  const bool owner = i < j;
  const V4<T>& a = owner ? p : q;
  const V4<T>& b = owner ? q : p;
  const Geo<T> g = pair_geo<T>(P, a, b);
  const bool stored = (mask >> s) & 1u;
  if (!(g.d2 < g.rs * g.rs)) {
    if (COMMIT && stored) hist[slot] = V2<T>{T(0), T(0)};  // contact opened: reset
    return;
  }
  const V4<T> w = fetch.v(j);
  const V4<T>& va = owner ? v : w;
  const V4<T>& vb = owner ? w : v;
  const V2<T> xi0 = stored ? hist[slot] : V2<T>{T(0), T(0)};
  const PairOut<T> o = pair_force<T>(P, g, a, va, b, vb, xi0);
  if (COMMIT) {
    const bool nz = (o.xi.x != T(0)) || (o.xi.y != T(0));
    if (nz || stored) hist[slot] = o.xi;
    nmask |= (nz ? 1u : 0u) << s;
  }
  if (owner) {
    fx.add(o.fx);
    fy.add(o.fy);
    diss += o.diss;
    un += o.un;
    ut += (MODE == kPeek && !primed) ? T(0) : o.ut;
  } else {
    fx.add(-o.fx);
    fy.add(-o.fy);
  }
  tq.add(p.z * o.cr);
}

// Symmetric 2x2 pseudo-inverse (eigen-decomposition, cutoff 2 eps sigma_max).
template <class T>
__device__ __forceinline__ V4<T> pinv_sym2_dev(T a, T b, T c) {
  const T eps = sizeof(T) == 4 ? T(1.1920929e-07) : T(2.220446049250313e-16);
  const T mean = T(0.5) * (a + c), half = T(0.5) * (a - c);
  const T rad = dev_sqrt(half * half + b * b);
  const T l1 = mean + rad, l2 = mean - rad;
  const T smax = fmax(fabs(l1), fabs(l2));
  const T cut = T(2) * eps * smax;
  if (fabs(l1) > cut && fabs(l2) > cut) {
    const T det = a * c - b * b;
    return V4<T>{c / det, -b / det, -b / det, a / det};
  }
  if (!(fabs(l1) > cut)) return V4<T>{T(0), T(0), T(0), T(0)};
  T vx, vy;
  if (fabs(b) > T(0)) {
    vx = l1 - c;
    vy = b;
  } else if (a >= c) {
    vx = T(1);
    vy = T(0);
  } else {
    vx = T(0);
    vy = T(1);
  }
  const T nv = dev_sqrt(vx * vx + vy * vy);
  vx /= nv;
  vy /= nv;
  return V4<T>{vx * vx / l1, vx * vy / l1, vx * vy / l1, vy * vy / l1};
}

// b - a of two discs through their cell origins (any order).
template <class T>
__device__ __forceinline__ V2<T> cell_delta(const Params<T>& P, const V4<T>& a, const V4<T>& b) {
  const int ca = lane_to_cell(a.w), cb = lane_to_cell(b.w);
  return V2<T>{fma((T)((cb & 0xFFFF) - (ca & 0xFFFF)), P.cell, b.x - a.x),
               fma((T)((cb >> 16) - (ca >> 16)), P.cell, b.y - a.y)};
}

// The shear invariant sqrt((E00 - E11)^2 + 4 E01^2) of the Green-Lagrange
// strain E = (G + G^T + G^T G) / 2, G = F - I, from the bond sums g and the
// pseudo-inverse pi of the reference-vector covariance.
template <class T>
__device__ __forceinline__ T shear_invariant(T g00, T g01, T g10, T g11, const V4<T>& pi) {
  const T f00 = g00 * pi.x + g01 * pi.z, f01 = g00 * pi.y + g01 * pi.w;
  const T f10 = g10 * pi.x + g11 * pi.z, f11 = g10 * pi.y + g11 * pi.w;
  const T e00 = T(0.5) * (T(2) * f00 + f00 * f00 + f10 * f10);
  const T e11 = T(0.5) * (T(2) * f11 + f01 * f01 + f11 * f11);
  const T e01 = T(0.5) * ((f01 + f10) + f00 * f01 + f10 * f11);
  const T dd = e00 - e11;
  return dev_sqrt(dd * dd + T(4) * (e01 * e01));
}

// Per-disc objective shear invariant over the disc's initial bonds (broken or
// not), the reference's local Green-Lagrange measure (dem.py:182-208) written
// with G = F - I: E = (G + G^T + G^T G) / 2.
template <class T, bool MULTI = false>
__global__ void strain_kernel(Params<T> P, Bufs<T> B) {
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const int n = MULTI ? B.ctl->n_live : P.n;
  if constexpr (!MULTI) {
    // One engine with bonds: the count, the own position, the pseudo-inverse
    // and every slot's word and reference vector in one round of loads (their
    // addresses are known up front), then all partner positions in a second
    // round, then the sums in slot order.
    const V4<T>* __restrict__ pos = B.pos[sp];
    const unsigned* __restrict__ bpart = B.bpart[lp];
    const V2<T>* __restrict__ bref = B.bref[lp];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int bc = B.bcnt[lp][i];
      const V4<T> p = pos[i];
      const V4<T> pi = B.bpinv[lp][i];
      unsigned w[kMaxBondSlots];
      V2<T> r[kMaxBondSlots];
#pragma unroll
      for (int u = 0; u < kMaxBondSlots; ++u) {
        if (u < P.BMAX) {
          w[u] = bpart[(size_t)u * n + i];
          r[u] = bref[(size_t)u * n + i];
        }
      }
      V4<T> q[kMaxBondSlots];
#pragma unroll
      for (int u = 0; u < kMaxBondSlots; ++u)
        if (u < bc) q[u] = pos[(int)(w[u] & kBondIdx)];
      T g00 = 0, g01 = 0, g10 = 0, g11 = 0;
#pragma unroll
      for (int u = 0; u < kMaxBondSlots; ++u) {
        if (u < bc) {
          const V2<T> cur = cell_delta<T>(P, p, q[u]);
          const T ux = cur.x - r[u].x, uy = cur.y - r[u].y;
          g00 += ux * r[u].x;
          g01 += ux * r[u].y;
          g10 += uy * r[u].x;
          g11 += uy * r[u].y;
        }
      }
      T sv = T(0);
      if (bc > 0) sv = shear_invariant<T>(g00, g01, g10, g11, pi);
      B.strain[i] = sv;
    }
  } else {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const int bc = B.bcnt[lp][i];
      T sv = T(0);
      if (bc > 0) {
        const Params<T>& Q = MULTI ? B.iparams[B.inst[lp][i]] : P;
        const V4<T>* pos = B.pos[sp];
        const V4<T> p = pos[i];
        T g00 = 0, g01 = 0, g10 = 0, g11 = 0;
        // four slots at a time: their slot words, then their partner positions,
        // then the sums (in slot order)
        constexpr int KS = 4;
        for (int s0 = 0; s0 < bc; s0 += KS) {
          unsigned w[KS];
#pragma unroll
          for (int u = 0; u < KS; ++u)
            if (s0 + u < bc) w[u] = B.bpart[lp][(size_t)(s0 + u) * P.n + i];
          V4<T> q[KS];
          V2<T> r[KS];
#pragma unroll
          for (int u = 0; u < KS; ++u) {
            if (s0 + u < bc) {
              q[u] = pos[(int)(w[u] & kBondIdx)];
              r[u] = B.bref[lp][(size_t)(s0 + u) * P.n + i];
            }
          }
#pragma unroll
          for (int u = 0; u < KS; ++u) {
            if (s0 + u < bc) {
              const V2<T> cur = cell_delta<T>(Q, p, q[u]);
              const T ux = cur.x - r[u].x, uy = cur.y - r[u].y;
              g00 += ux * r[u].x;
              g01 += ux * r[u].y;
              g10 += uy * r[u].x;
              g11 += uy * r[u].y;
            }
          }
        }
        sv = shear_invariant<T>(g00, g01, g10, g11, B.bpinv[lp][i]);
      }
      B.strain[i] = sv;
    }
  }
}

// Pipelined strain for FP32 engines: a persistent grid in which each thread
// stages its next disc's first round (count, own position, pseudo-inverse,
// slot words, reference vectors) into shared memory with cp.async while it
// gathers the current disc's partners and sums its bonds. The same sums in
// the same order as strain_kernel. Layout [stage][slot][thread].
constexpr int kStrainBlock = 256;
constexpr size_t kStrainSmem = (size_t)2 * kStrainBlock * (kMaxBondSlots * (4 + 8) + 16 + 16 + 4);

template <class T>
__global__ void __launch_bounds__(kStrainBlock) strain_kernel_async(Params<T> P, Bufs<T> B) {
  static_assert(sizeof(T) == 4, "the pipelined strain serves FP32 engines");
  using bulk::cp16;
  using bulk::cp4;
  using bulk::cp8;
  using bulk::cp_commit;
  using bulk::cp_wait;
  constexpr int BL = kStrainBlock, S = kMaxBondSlots;
  extern __shared__ uint4 strain_smem[];
  V4<T>* spos = reinterpret_cast<V4<T>*>(strain_smem);              // [2][BL]
  V4<T>* spi = spos + 2 * BL;                                        // [2][BL]
  V2<T>* sref = reinterpret_cast<V2<T>*>(spi + 2 * BL);              // [2][S][BL]
  unsigned* sw = reinterpret_cast<unsigned*>(sref + 2 * S * BL);     // [2][S][BL]
  int* sbc = reinterpret_cast<int*>(sw + 2 * S * BL);                // [2][BL]
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const int n = P.n, BM = P.BMAX;
  const int t = threadIdx.x;
  const int stride = gridDim.x * BL;
  const V4<T>* __restrict__ pos = B.pos[sp];
  const unsigned* __restrict__ bpart = B.bpart[lp];
  const V2<T>* __restrict__ bref = B.bref[lp];
  auto stage = [&](int i, int st) {
    cp4(sbc + st * BL + t, B.bcnt[lp] + i);
    cp16(spos + st * BL + t, pos + i);
    cp16(spi + st * BL + t, B.bpinv[lp] + i);
#pragma unroll
    for (int u = 0; u < S; ++u) {
      if (u < BM) {
        const size_t k = (size_t)u * n + i;
        cp4(sw + (st * S + u) * BL + t, bpart + k);
        cp8(sref + (st * S + u) * BL + t, bref + k);
      }
    }
  };
  int i = blockIdx.x * BL + t;
  if (i < n) stage(i, 0);
  cp_commit();
  for (int st = 0; i < n; i += stride, st ^= 1) {
    const int i1 = i + stride;
    if (i1 < n) stage(i1, st ^ 1);
    cp_commit();
    cp_wait<1>();  // this disc's staged loads have landed
    const int bc = sbc[st * BL + t];
    const V4<T> p = spos[st * BL + t];
    V4<T> q[S];
#pragma unroll
    for (int u = 0; u < S; ++u)
      if (u < bc) q[u] = pos[(int)(sw[(st * S + u) * BL + t] & kBondIdx)];
    T g00 = 0, g01 = 0, g10 = 0, g11 = 0;
#pragma unroll
    for (int u = 0; u < S; ++u) {
      if (u < bc) {
        const V2<T> r = sref[(st * S + u) * BL + t];
        const V2<T> cur = cell_delta<T>(P, p, q[u]);
        const T ux = cur.x - r.x, uy = cur.y - r.y;
        g00 += ux * r.x;
        g01 += ux * r.y;
        g10 += uy * r.x;
        g11 += uy * r.y;
      }
    }
    T sv = T(0);
    if (bc > 0) sv = shear_invariant<T>(g00, g01, g10, g11, spi[st * BL + t]);
    B.strain[i] = sv;
  }
  cp_wait<0>();
}

// Per-thread ledger terms of the particles a thread processed.
template <class T>
struct ThreadLedger {
  float vmax2 = 0.0f;
  T diss = T(0), un = T(0), ut = T(0);
  T ub = T(0), frac = T(0);   // bond elastic energy, fracture release
  T ifx = T(0), ify = T(0);  // indenter force on this thread's discs
  int broke = 0;
  double ke = 0.0, pe = 0.0;
  bool bad = false;
};

// The break test `strain > eps * strength` decided as in FP64. FP32: the
// threshold lies in [lo, hi] = [eps_lo * strength rounded down, eps_hi *
// strength rounded up], so a strain outside that bracket is decided in FP32
// with the FP64 answer; only a strain inside it is compared in FP64.
template <class T>
__device__ __noinline__ bool exceeds_fp64(T strain, double eps, T strength) {
  return (double)strain > eps * (double)strength;
}

template <class T>
__device__ __forceinline__ bool exceeds(T strain, double eps, float eps_lo, float eps_hi, T strength) {
  if constexpr (sizeof(T) == 4) {
    const float hi = __fmul_ru(eps_hi, strength);
    if (strain > hi) return true;
    const float lo = __fmul_rd(eps_lo, strength);
    if (strain <= lo) return false;
    // rare: the strain sits within a float ulp of the threshold (kept out of
    // line so that no FP64 conversion is hoisted onto the common path)
    return exceeds_fp64<T>(strain, eps, strength);
  } else {
    return (double)strain > eps * (double)strength;
  }
}

// One bond slot s of disc i: the break test (FP64 comparison of the strains
// against the bond's thresholds), then the bond law while intact, or the Hertz
// contact with the slot's history once broken (dem.py:243-292 semantics: a
// bond broken at this evaluation already acts as a contact).
// Loads of one bond slot, issued for a few slots together before any of
// them is computed (the partner index comes from the slot word).
template <class T>
struct BondIn {
  unsigned w;   // slot word: partner | mode | broken
  V4<T> q, wv;  // partner position, velocity
  V2<T> rs;     // reference vector (stored for the slot's own side)
  V2<T> us;     // shear displacement / contact history
  T sf;         // strength factor
  T sj;         // partner's objective shear strain
};

template <class T, int MODE, class A>
__device__ __forceinline__ void do_bond(const Params<T>& P, const Bufs<T>& B, int lp, int i, size_t k,
                                        long long eval, const V4<T>& p, const V4<T>& v, const BondIn<T>& in,
                                        T si, A& fx, A& fy, A& tq, ThreadLedger<T>& L,
                                        int primed) {
  constexpr bool COMMIT = MODE != kPeek;
  const unsigned w = in.w;
  const int j = (int)(w & kBondIdx);
  const V4<T>& q = in.q;
  const V4<T>& wv = in.wv;
  const bool owner = i < j;
  const V4<T>& a = owner ? p : q;
  const V4<T>& b = owner ? q : p;
  const V4<T>& va = owner ? v : wv;
  const V4<T>& vb = owner ? wv : v;
  const V2<T> rs = in.rs;
  const V2<T> ref = owner ? rs : V2<T>{-rs.x, -rs.y};
  const Geo<T> g = pair_geo<T>(P, a, b);
  bool broken = (w & kBondBroken) != 0u;
  V2<T> us = in.us;
  if (!broken) {
    const T ux = g.dx - ref.x, uy = g.dy - ref.y;
    // FP32: bond lengths and directions from rsqrt / rcp (a few ulp; the
    // extension is formed without cancellation); FP64: exact operations
    T d, l0, inv_d, inv_l0, inv_dl;
    if constexpr (sizeof(T) == 4) {
      // _rn intrinsics are never fused into an FMA, so every kernel that
      // inlines this computes the same bits
      inv_d = rsqrtf(g.d2);
      d = __fmul_rn(g.d2, inv_d);
      const T l02 = __fadd_rn(__fmul_rn(ref.x, ref.x), __fmul_rn(ref.y, ref.y));
      inv_l0 = rsqrtf(l02);
      l0 = __fmul_rn(l02, inv_l0);
      inv_dl = __frcp_rn(__fadd_rn(d, l0));
    } else {
      d = dev_sqrt(g.d2);
      l0 = dev_sqrt(ref.x * ref.x + ref.y * ref.y);
      inv_d = T(1) / d;
      inv_l0 = T(1) / l0;
      inv_dl = T(1) / (d + l0);
    }
    const T ext = sizeof(T) == 4 ? (T(2) * (ref.x * ux + ref.y * uy) + (ux * ux + uy * uy)) * inv_dl
                                 : (T(2) * (ref.x * ux + ref.y * uy) + (ux * ux + uy * uy)) / (d + l0);
    const T tensile = sizeof(T) == 4 ? ext * inv_l0 : ext / l0;
    const T shear = T(0.5) * (si + in.sj);
    const T sf = in.sf;
    const bool bt = exceeds<T>(tensile, P.eps_t, P.eps_t_lo, P.eps_t_hi, sf);
    const bool bs = exceeds<T>(shear, P.eps_s, P.eps_s_lo, P.eps_s_hi, sf);
    if (bt || bs) {
      broken = true;
      if (owner) {
        // spring energy released, minus the Hertz energy a still-overlapping
        // pair acquires as a contact at once (dem.py:270-277 books both)
        const T ov = fmax(g.rs - d, T(0));
        const T acquired = T(0.4) * (T(2) / T(3)) * P.estar2 * dev_sqrt(a.z * b.z / g.rs * ov) * ov * ov;
        L.frac += T(0.5) * P.kn * ext * ext + T(0.5) * P.ks * (us.x * us.x + us.y * us.y) - acquired;
        L.broke += 1;
      }
      if (COMMIT) {
        const unsigned mode = (bt ? 1u : 0u) | (bs ? 2u : 0u);
        B.bpart[lp][k] = (w & kBondIdx) | (mode << kBondModeShift) | kBondBroken;
        B.bfail[lp][k] = (int)eval;
      }
      us = V2<T>{T(0), T(0)};  // the contact starts without tangential history
    } else if (va.w + vb.w > T(0)) {
      const T nx = sizeof(T) == 4 ? g.dx * inv_d : g.dx / d;
      const T ny = sizeof(T) == 4 ? g.dy * inv_d : g.dy / d;
      const T wsum = va.z * a.z + vb.z * b.z;
      const T vrx = (va.x - vb.x) - wsum * ny;
      const T vry = (va.y - vb.y) + wsum * nx;
      const T vn = vrx * nx + vry * ny;
      const T vtx = vrx - vn * nx, vty = vry - vn * ny;
      T sx = us.x + vtx * P.dt, sy = us.y + vty * P.dt;
      const T sn = sx * nx + sy * ny;
      sx -= sn * nx;
      sy -= sn * ny;
      T cn, cs;
      if constexpr (sizeof(T) == 4) {
        const T rm = rsqrtf(va.w + vb.w);  // sqrt(m*)
        cn = P.cn_k * rm;
        cs = P.cs_k * rm;
      } else {
        const T meff = T(1) / (va.w + vb.w);
        cn = T(2) * P.bzeta * dev_sqrt(P.kn * meff);
        cs = T(2) * P.bzeta * dev_sqrt(P.ks * meff);
      }
      const T fnm = P.kn * ext - cn * vn;
      const T fax = fnm * nx - P.ks * sx - cs * vtx;
      const T fay = fnm * ny - P.ks * sy - cs * vty;
      const T cr = nx * fay - ny * fax;
      if (owner) {
        fx.add(fax);
        fy.add(fay);
        L.diss += (cn * vn * vn + cs * (vtx * vtx + vty * vty)) * P.dt;
        L.ub += T(0.5) * P.kn * ext * ext + T(0.5) * P.ks * (sx * sx + sy * sy);
      } else {
        fx.add(-fax);
        fy.add(-fay);
      }
      tq.add(p.z * cr);
      if (COMMIT) B.bus[lp][k] = V2<T>{sx, sy};
      return;
    } else {
      return;  // intact bond between two clamped discs
    }
  }
  // broken: Hertz-Mindlin contact with the slot's history
  const bool stored = (us.x != T(0)) || (us.y != T(0));
  if (!(g.d2 < g.rs * g.rs)) {
    if (COMMIT && stored) B.bus[lp][k] = V2<T>{T(0), T(0)};
    return;
  }
  const PairOut<T> o = pair_force<T>(P, g, a, va, b, vb, us);
  if (COMMIT) B.bus[lp][k] = o.xi;
  if (owner) {
    fx.add(o.fx);
    fy.add(o.fy);
    L.diss += o.diss;
    L.un += o.un;
    L.ut += (MODE == kPeek && !primed) ? T(0) : o.ut;
  } else {
    fx.add(-o.fx);
    fy.add(-o.fy);
  }
  tq.add(p.z * o.cr);
}

// Rigid circular indenter, Hertz normal + Tsuji dashpot, frictionless
// (the reference's tool, dem.py:294-312, with the Hertz law of the contacts).
// Distances in FP64 from the integer cell origin, only for discs near it.
template <class T, class A>
__device__ __forceinline__ void indenter_contact(const Params<T>& P, long long eval, const V4<T>& p, const V4<T>& v,
                                                 A& fx, A& fy, ThreadLedger<T>& L) {
  const int c = lane_to_cell(p.w);
  {
    // FP32 screen: a disc clearly out of reach never touches FP64 (the FP32
    // positions carry ~1e-7 relative error; the margin is 1e-5 relative)
    const float ef = (float)(int)eval;  // evaluation counts stay far below 2^31
    const float cxf = P.ind_x0f + ef * P.ind_dxf, cyf = P.ind_y0f + ef * P.ind_dyf;
    const float xf = (float)(c & 0xFFFF) * (float)P.cell + (float)p.x;
    const float yf = (float)(c >> 16) * (float)P.cell + (float)p.y;
    const float reachf = (float)P.irad + (float)p.z;
    const float dxf = fabsf(xf - cxf), dyf = fabsf(yf - cyf);
    const float margin =
        1e-5f * (fabsf(xf) + fabsf(yf) + fabsf(cxf) + fabsf(cyf) + reachf + ef * (fabsf(P.ind_dxf) + fabsf(P.ind_dyf)));
    if (dxf >= reachf + margin || dyf >= reachf + margin) return;
  }
  const double t = (double)eval * (double)P.dt;
  const double cx = P.ind_x0 + t * P.ind_vx, cy = P.ind_y0 + t * P.ind_vy;
  const double x = (double)(c & 0xFFFF) * (double)P.cell + (double)p.x;
  const double y = (double)(c >> 16) * (double)P.cell + (double)p.y;
  const double dx = x - cx, dy = y - cy;
  const double R = (double)P.irad, r = (double)p.z;
  const double reach = R + r;
  if (fabs(dx) >= reach || fabs(dy) >= reach) return;
  const double dd = sqrt(dx * dx + dy * dy);
  const double delta = reach - dd;
  if (!(delta > 0.0) || !(v.w > T(0))) return;
  const double nx = dx / dd, ny = dy / dd;
  const double reff = R * r / reach;
  const double sq = sqrt(reff * delta);
  const double sn = 2.0 * ((double)P.estar2 * 0.5) * sq;
  const double fel = (2.0 / 3.0) * sn * delta;
  const double vapp = -(((double)v.x - P.ind_vx) * nx + ((double)v.y - P.ind_vy) * ny);
  const double m = 1.0 / (double)v.w;
  const double fn = fmax(fel + (double)P.damp * sqrt(sn * m) * vapp, 0.0);
  fx.add((T)(fn * nx));
  fy.add((T)(fn * ny));
  L.ifx += (T)(fn * nx);
  L.ify += (T)(fn * ny);
  L.diss += (T)((fn - fel) * vapp * (double)P.dt);
  L.un += (T)(0.4 * fel * delta);
}

// Compensated FP32 coordinates (Params::prem): a coordinate is the pair
// (x, r) with x the FP32 offset and r the FP32 remainder of its rounding.
// a + b == s + e exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (x, r) += a * b, renormalised so that |r| stays within half an ulp of the
// returned offset: the product's rounding error (from an FMA) and the sum's
// (TwoSum) go to the remainder instead of being lost.
__device__ __forceinline__ float add_prod_comp(float x, float& r, float a, float b) {
  const float d = __fmul_rn(a, b);
  const float de = __fmaf_rn(a, b, -d);
  float s, e;
  two_sum(x, d, s, e);
  const float t = __fadd_rn(__fadd_rn(r, e), de);
  float s2, r2;
  two_sum(s, t, s2, r2);
  r = r2;
  return s2;
}

// Everything one particle does in one evaluation: its candidate slots, the
// walls, and (committing modes) the velocity-Verlet update into the other
// buffers. p, v, hd are the particle's own loads (already issued).
// Positions of the first three partners of a list head, issued together.
template <class T, class F>
__device__ __forceinline__ void load_head_partners(const F& fetch, const uint4& hd, V4<T>& q0, V4<T>& q1,
                                                   V4<T>& q2) {
  const int cnt = (int)(hd.x & 0xFFu);
  if (cnt > 0) q0 = fetch.p((int)hd.y);
  if (cnt > 1) q1 = fetch.p((int)hd.z);
  if (cnt > 2) q2 = fetch.p((int)hd.w);
}

// process_particle with the first three partners' positions already loaded.
// rem_pre: the disc's position remainder when the caller has it already
// (null: loaded here). PREW: the caller has staged the disc's bond slot
// words (pw[u * pw_stride]), bond count and strain.
template <class T, int MODE, bool FEAT, class F, bool S64 = false, bool PREW = false>
__device__ __forceinline__ void process_particle_q(const Params<T>& P, const Bufs<T>& B, const F& fetch, int sp,
                                                   int lp, int i, const V4<T>& p, const V4<T>& v, const uint4& hd,
                                                   const V4<T>& q0, const V4<T>& q1, const V4<T>& q2, int primed,
                                                   long long eval, ThreadLedger<T>& L,
                                                   const float2* rem_pre = nullptr, const unsigned* pw = nullptr,
                                                   int pw_stride = 0, int pbc = 0, T psi = T(0)) {
  constexpr bool COMMIT = MODE != kPeek;
  const int n = P.n;
  const unsigned* __restrict__ tail = B.nbr[lp];
  V2<T>* __restrict__ hist = B.hist[lp];
  const int cnt = (int)(hd.x & 0xFFu);
  // the position remainder, loaded now and used after the contact loop
  float2 rem = make_float2(0.0f, 0.0f);
  if constexpr (sizeof(T) == 4) {
    if (P.prem) rem = rem_pre ? *rem_pre : B.prem[lp][i];
  }
  const unsigned mask = hd.x >> 8;
  unsigned nmask = 0u;
  typename AccSel<T, S64>::type fx, fy, tq;
  if (FEAT && P.BMAX > 0) {
    // the count and every slot word in one round of loads (slots past the
    // count are allocated, their words unused)
    unsigned wds[kMaxBondSlots];
#pragma unroll
    for (int u = 0; u < kMaxBondSlots; ++u)
      if (u < P.BMAX) wds[u] = PREW ? pw[u * pw_stride] : B.bpart[lp][(size_t)u * n + i];
    const int bc = PREW ? pbc : B.bcnt[lp][i];
    if (bc > 0) {
      const T si = PREW ? psi : B.strain[i];
      constexpr int KB = 2;  // bond slots whose partner loads are in flight together
#pragma unroll
      for (int s0 = 0; s0 < kMaxBondSlots; s0 += KB) {
        if (s0 >= bc) break;
        BondIn<T> in[KB];
#pragma unroll
        for (int u = 0; u < KB; ++u) in[u].w = wds[s0 + u];
#pragma unroll
        for (int u = 0; u < KB; ++u) {
          if (s0 + u < bc) {
            const size_t k = (size_t)(s0 + u) * n + i;
            const int j = (int)(in[u].w & kBondIdx);
            in[u].q = fetch.p(j);
            in[u].wv = fetch.v(j);
            in[u].sj = B.strain[j];
            in[u].rs = B.bref[lp][k];
            in[u].us = B.bus[lp][k];
            in[u].sf = B.bstr[lp][k];
          }
        }
#pragma unroll
        for (int u = 0; u < KB; ++u)
          if (s0 + u < bc)
            do_bond<T, MODE>(P, B, lp, i, (size_t)(s0 + u) * n + i, eval, p, v, in[u], si, fx, fy, tq, L, primed);
      }
    }
  }
  if (cnt > 0)
    do_slot<T, MODE>(P, fetch, hist, i, (int)hd.y, 0, (size_t)i, p, v, q0, mask, nmask, fx, fy, tq, L.diss, L.un,
                     L.ut, primed);
  if (cnt > 1)
    do_slot<T, MODE>(P, fetch, hist, i, (int)hd.z, 1, (size_t)n + i, p, v, q1, mask, nmask, fx, fy, tq, L.diss,
                     L.un, L.ut, primed);
  if (cnt > 2)
    do_slot<T, MODE>(P, fetch, hist, i, (int)hd.w, 2, (size_t)2 * n + i, p, v, q2, mask, nmask, fx, fy, tq, L.diss,
                     L.un, L.ut, primed);
  for (int s = kHeadSlots; s < cnt; ++s) {
    const int j = (int)tail[(size_t)(s - kHeadSlots) * n + i];
    const V4<T> q = fetch.p(j);
    do_slot<T, MODE>(P, fetch, hist, i, j, s, (size_t)s * n + i, p, v, q, mask, nmask, fx, fy, tq, L.diss, L.un,
                     L.ut, primed);
  }
  if (COMMIT && nmask != mask) B.head[lp][i].x = (hd.x & 0xFFu) | (nmask << 8);
  const int c = lane_to_cell(p.w);
  if (FEAT && P.irad > T(0)) indenter_contact<T>(P, eval, p, v, fx, fy, L);
  if (P.walls && v.w > T(0)) {
    const int cx = c & 0xFFFF, cy = c >> 16;
    if ((cx == 0 || cx == P.ncx - 1 || cy == 0 || cy == P.ncy - 1)) {
      V2<T>* wh = B.whist[lp];
      const bool old_xi = (MODE == kPeek && !primed);
      if ((P.walls & 1) && cx == 0)
        wall_contact<T, COMMIT>(P, T(1), T(0), p.x, p, v, &wh[i], fx, fy, tq, L.diss, L.un, L.ut, old_xi);
      if ((P.walls & 2) && cx == P.ncx - 1)
        wall_contact<T, COMMIT>(P, T(-1), T(0), P.cell - p.x, p, v, &wh[(size_t)n + i], fx, fy, tq, L.diss, L.un,
                                L.ut, old_xi);
      if ((P.walls & 4) && cy == 0)
        wall_contact<T, COMMIT>(P, T(0), T(1), p.y, p, v, &wh[(size_t)2 * n + i], fx, fy, tq, L.diss, L.un, L.ut,
                                old_xi);
      if ((P.walls & 8) && cy == P.ncy - 1)
        wall_contact<T, COMMIT>(P, T(0), T(-1), P.cell - p.y, p, v, &wh[(size_t)3 * n + i], fx, fy, tq, L.diss,
                                L.un, L.ut, old_xi);
    }
  }
  const T Fx = fx.get(), Fy = fy.get(), Tz = tq.get();
  const T inv_m = v.w;  // 0 for a clamped disc
  const bool free = inv_m > T(0);
  const T inv_i = inv_m * P.kinv / (p.z * p.z);
  const T ax = free ? Fx * inv_m + P.gx : T(0);
  const T ay = free ? Fy * inv_m + P.gy : T(0);
  const T al = Tz * inv_i;
  if (MODE == kPeek) {
    const T h = primed ? P.half_dt : T(0);
    const T vx = v.x + h * ax, vy = v.y + h * ay, om = v.z + h * al;
    B.peek_vel[i] = V4<T>{vx, vy, om, T(0)};
    B.peek_force[i] = free ? V4<T>{Fx + P.gx / inv_m, Fy + P.gy / inv_m, Tz, T(0)} : V4<T>{Fx, Fy, Tz, T(0)};
    // energies in FP64: the potential needs absolute positions
    if (free) {
      const double m = 1.0 / (double)inv_m;
      const double r = (double)p.z;
      L.ke += 0.5 * m * ((double)vx * vx + (double)vy * vy) + 0.5 * (m * r * r / (double)P.kinv) * (double)om * om;
      const double x = (double)(c & 0xFFFF) * (double)P.cell + (double)p.x + (double)rem.x;
      const double y = (double)(c >> 16) * (double)P.cell + (double)p.y + (double)rem.y;
      L.pe += -m * ((double)P.gx * x + (double)P.gy * y);
    }
    // The contact, bond and indenter energies above are those of the FP32
    // offsets; the remainder moves the disc by r, which changes them to first
    // order by -F . r (F: the disc's force without gravity). Counted with
    // the potential energy.
    if (sizeof(T) == 4 && P.prem) L.pe -= (double)Fx * (double)rem.x + (double)Fy * (double)rem.y;
  } else {
    T vx, vy, om;
    if (MODE == kPrime || (MODE == kBatch && !primed)) {
      vx = v.x + P.half_dt * ax;
      vy = v.y + P.half_dt * ay;
      om = v.z + P.half_dt * al;
    } else {
      vx = (v.x + P.half_dt * ax) + P.half_dt * ax;
      vy = (v.y + P.half_dt * ay) + P.half_dt * ay;
      om = (v.z + P.half_dt * al) + P.half_dt * al;
    }
    T ox, oy;
    if (sizeof(T) == 4 && P.prem) {
      float2 r = rem;
      ox = (T)add_prod_comp((float)p.x, r.x, (float)P.dt, (float)vx);
      oy = (T)add_prod_comp((float)p.y, r.y, (float)P.dt, (float)vy);
      B.prem[lp][i] = r;
    } else {
      ox = p.x + P.dt * vx;
      oy = p.y + P.dt * vy;
    }
    B.pos[sp ^ 1][i] = V4<T>{ox, oy, p.z, p.w};
    B.vel[sp ^ 1][i] = V4<T>{vx, vy, om, v.w};
    L.vmax2 = fmaxf(L.vmax2, (float)(vx * vx + vy * vy));
    if (!(isfinite(ox) && isfinite(oy) && isfinite(vx) && isfinite(vy) && isfinite(om))) L.bad = true;
  }
}

template <class T, int MODE, bool FEAT, bool S64 = false>
__device__ __forceinline__ void process_particle(const Params<T>& P, const Bufs<T>& B, int sp, int lp, int i,
                                                 const V4<T>& p, const V4<T>& v, const uint4& hd, int primed,
                                                 long long eval, ThreadLedger<T>& L,
                                                 const float2* rem_pre = nullptr) {
  V4<T> q0{}, q1{}, q2{};
  const GlobalFetch<T> fetch{B.pos[sp], B.vel[sp]};
  load_head_partners<T>(fetch, hd, q0, q1, q2);
  process_particle_q<T, MODE, FEAT, GlobalFetch<T>, S64>(P, B, fetch, sp, lp, i, p, v, hd, q0, q1, q2, primed, eval, L,
                                                         rem_pre);
}

// Control fields a step kernel reads once at its start. disp and target are
// written only by the last warp of the kernel, after every block has read
// them, so the epilogue needs no second round trip for them.
struct StepCtl {
  int sp, lp;
  long long evals, target;
  float disp;
};

// Buffer parities and evaluation count of a launch when the host knows them
// (plain launches after a host read of the control block): the launch's own
// state loads then need not wait for the control block's cold read.
struct StepHint {
  int valid, sp, lp;
  long long evals;
};

__device__ __forceinline__ StepCtl load_step_ctl(const Ctl* ctl, const StepHint& hint = StepHint{0, 0, 0, 0}) {
  StepCtl c;
  if (hint.valid) {
    c.sp = hint.sp;
    c.lp = hint.lp;
    c.evals = hint.evals;
  } else {
    c.sp = ctl->sp;
    c.lp = ctl->lp;
    c.evals = ctl->evals;
  }
  c.target = ctl->target;  // read only by the last block's bookkeeping
  c.disp = ctl->disp;
  return c;
}

// Commit epilogue: per-warp ledger partials (fire-and-forget adds; one
// warp owns each slot, so every slot still sums its steps in step order),
// the block's speed bound, then the last block of the grid does the step
// bookkeeping (indenter reaction, rebuild trigger) and sets the graph's
// conditions. Its tail costs two round trips to L2: the grid ticket and one
// 8-byte read of the speed bound with the status word.
template <class T, bool FEAT>
__device__ __forceinline__ void commit_epilogue(const Params<T>& P, const Bufs<T>& B, const StepCtl& c,
                                                const ThreadLedger<T>& L, cudaGraphConditionalHandle h_rebuild,
                                                cudaGraphConditionalHandle h_loop, int use_cond) {
  const int sp = c.sp;
  Ctl* ctl = B.ctl;
  float wm = L.vmax2;
  T wd = L.diss, wf = L.frac, wix = L.ifx, wiy = L.ify;
  int wb = L.broke;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, off));
    wd += __shfl_xor_sync(0xffffffffu, wd, off);
    if (FEAT) {
      wf += __shfl_xor_sync(0xffffffffu, wf, off);
      wix += __shfl_xor_sync(0xffffffffu, wix, off);
      wiy += __shfl_xor_sync(0xffffffffu, wiy, off);
      wb += __shfl_xor_sync(0xffffffffu, wb, off);
    }
  }
  __shared__ float s_vmax[32];
  if ((threadIdx.x & 31) == 0) {
    const size_t gw = (size_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (wd != T(0)) atomicAdd(&B.diss_part[gw], (double)wd);
    if (FEAT && wf != T(0)) atomicAdd(&B.frac_part[gw], (double)wf);
    if (FEAT && wb) atomicAdd(&ctl->broken, wb);
    if (FEAT && (wix != T(0) || wiy != T(0))) {
      const unsigned e = atomicAdd(&ctl->load_entries, 1u);
      B.ind_part[3 * (size_t)e] = (double)gw;
      B.ind_part[3 * (size_t)e + 1] = (double)wix;
      B.ind_part[3 * (size_t)e + 2] = (double)wiy;
    }
    s_vmax[threadIdx.x >> 5] = wm;
  }
  const int bad = __syncthreads_or(L.bad ? 1 : 0);
  // with an indenter the whole last block puts the reaction partials in order
  const bool ind = FEAT && P.irad > T(0);
  if (!ind && threadIdx.x >= 32) return;
  __shared__ unsigned s_last;
  bool last = false;
  if (threadIdx.x < 32) {
    // the block's speed bound: warp 0 reduces the warps' bounds (>= 0)
    float bm = threadIdx.x < (blockDim.x >> 5) ? s_vmax[threadIdx.x] : 0.0f;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, off));
    if (threadIdx.x == 0) {
      if (bad) atomicOr(&ctl->status, (int)kStatusNonfinite);
      atomicMax(&ctl->vmax2_bits, __float_as_uint(bm));
      // the grid ticket with release-acquire order: this block's writes (its
      // threads' through the barrier above) are visible before its ticket,
      // and the last block sees every other block's writes after its own
      unsigned t;
      asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(t) : "l"(&ctl->ticket) : "memory");
      last = t == gridDim.x - 1;
      s_last = last ? 1u : 0u;
    }
  }
  if (ind) {
    __syncthreads();
    if (!s_last) return;
    // the indenter partials (warp id, fx, fy), one per warp that touched the
    // indenter, put in warp order by rank (the keys are distinct) into the
    // second half of ind_part, by every thread of the last block
    const unsigned m = *reinterpret_cast<volatile unsigned*>(&ctl->load_entries);
    const double* e = B.ind_part;
    double* o = B.ind_part + 3 * (size_t)P.ind_slots;
    for (unsigned a = threadIdx.x; a < m; a += blockDim.x) {
      const double k0 = e[3 * a];
      unsigned r = 0;
      for (unsigned u = 0; u < m; ++u) r += (e[3 * u] < k0) ? 1u : 0u;
      o[3 * r] = k0;
      o[3 * r + 1] = e[3 * a + 1];
      o[3 * r + 2] = e[3 * a + 2];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    // summed in warp order, eight loads in flight at a time
    double sx = 0.0, sy = 0.0;
    unsigned a = 0;
    for (; a + 8 <= m; a += 8) {
      double x[8], y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        x[u] = o[3 * (a + u) + 1];
        y[u] = o[3 * (a + u) + 2];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        sx += x[u];
        sy += y[u];
      }
    }
    for (; a < m; ++a) {
      sx += o[3 * a + 1];
      sy += o[3 * a + 2];
    }
    ctl->reaction_x = -sx;
    ctl->reaction_y = -sy;
    ctl->tool_work += (double)P.dt * (sx * P.ind_vx + sy * P.ind_vy);
    if (c.evals < (long long)P.load_cap) {
      B.load[2 * c.evals] = -sx;
      B.load[2 * c.evals + 1] = -sy;
    }
    ctl->load_entries = 0u;
  } else if (!last) {
    return;
  }
  const unsigned long long pair = *reinterpret_cast<volatile unsigned long long*>(&ctl->vmax2_bits);
  const unsigned vbits = (unsigned)(pair & 0xFFFFFFFFull);
  const int status = (int)(pair >> 32);
  const float vmax = sqrtf(__uint_as_float(vbits));
  ctl->vmax2_bits = 0u;
  ctl->ticket = 0;
  ctl->sp = sp ^ 1;
  const long long evals = c.evals + 1;
  ctl->evals = evals;
  const float disp = c.disp + vmax * (float)P.dt;
  ctl->disp = disp;
  const int rebuild = (disp > P.rebuild_disp) ? 1 : 0;
  ctl->rebuild_pending = rebuild;
  // a non-finite state or a bounded wait that ran out ends the step loop
  const int keep_going = (evals < c.target) && !(status & (kStatusNonfinite | kStatusTimeout));
  // use_cond bit 0: this launch sits in a graph with a rebuild IF node;
  // bit 1: it also sits in the step loop's WHILE body
  if (use_cond & 1) cudaGraphSetConditional(h_rebuild, (unsigned)rebuild);
  if (use_cond & 2) cudaGraphSetConditional(h_loop, (unsigned)keep_going);
}

// One thread per particle (variant 0) and the read-back kernel.
template <class T, int MODE, bool FEAT, bool S64 = false>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 4 : 2) force_kernel(Params<T> P, Bufs<T> B,
                                                            cudaGraphConditionalHandle h_rebuild,
                                                            cudaGraphConditionalHandle h_loop, int use_cond,
                                                            int primed, StepHint hint) {
  const StepCtl c = load_step_ctl(B.ctl, hint);
  const int sp = c.sp, lp = c.lp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  ThreadLedger<T> L;
  if (i < P.n) {
    const V4<T> p = B.pos[sp][i];
    const V4<T> v = B.vel[sp][i];
    const uint4 hd = B.head[lp][i];
    process_particle<T, MODE, FEAT, S64>(P, B, sp, lp, i, p, v, hd, primed, c.evals, L);
  }
  if (MODE == kPeek) {
    const double k = block_sum_d(L.ke);
    const double g = block_sum_d(L.pe);
    const double a = block_sum_t<T>(L.un);
    const double b = block_sum_t<T>(L.ut);
    const double d = block_sum_t<T>(primed ? L.diss : T(0));
    const double ub = block_sum_t<T>(L.ub);
    const double fr = block_sum_t<T>(L.frac);
    const double tw = block_sum_t<T>((L.ifx * (T)P.ind_vx + L.ify * (T)P.ind_vy) * P.dt);
    const double nb = block_sum_t<T>((T)L.broke);
    if (threadIdx.x == 0) {
      double* o = B.peek_part + (size_t)blockIdx.x * 12;
      o[0] = k;
      o[1] = g;
      o[2] = a;
      o[3] = b;
      o[4] = d;
      o[5] = ub;
      o[6] = fr;
      o[7] = tw;
      o[8] = nb;
    }
    return;
  }
  commit_epilogue<T, FEAT>(P, B, c, L, h_rebuild, h_loop, use_cond);
}

// Persistent grid-stride variant: while a thread works on particle i it has
// the loads of its next particle already in flight (twice the memory-level
// parallelism of variant 0 at the cost of a dozen registers).
template <class T, int MODE, int BLOCK, int MINB, bool FEAT, bool S64 = false>
__global__ void __launch_bounds__(BLOCK, MINB) force_kernel_pf(Params<T> P, Bufs<T> B,
                                                               cudaGraphConditionalHandle h_rebuild,
                                                               cudaGraphConditionalHandle h_loop, int use_cond,
                                                               int primed, StepHint hint) {
  static_assert(MODE != kPeek, "read-back uses force_kernel");
  const StepCtl c = load_step_ctl(B.ctl, hint);
  const int sp = c.sp, lp = c.lp;
  const long long eval = c.evals;
  const int stride = gridDim.x * BLOCK;
  int i = blockIdx.x * BLOCK + threadIdx.x;
  ThreadLedger<T> L;
  V4<T> p{}, v{};
  uint4 hd = make_uint4(0u, 0u, 0u, 0u);
  // the position remainder travels with the own state (FP32 engines)
  const bool pr = sizeof(T) == 4 && P.prem;
  float2 r{0.0f, 0.0f};
  if (i < P.n) {
    p = B.pos[sp][i];
    v = B.vel[sp][i];
    hd = B.head[lp][i];
    if (pr) r = B.prem[lp][i];
  }
  while (i < P.n) {
    const int nx = i + stride;
    V4<T> pn{}, vn{};
    uint4 hn = make_uint4(0u, 0u, 0u, 0u);
    float2 rn{0.0f, 0.0f};
    if (nx < P.n) {
      pn = B.pos[sp][nx];
      vn = B.vel[sp][nx];
      hn = B.head[lp][nx];
      if (pr) rn = B.prem[lp][nx];
    }
    process_particle<T, MODE, FEAT, S64>(P, B, sp, lp, i, p, v, hd, primed, eval, L, &r);
    i = nx;
    p = pn;
    v = vn;
    hd = hn;
    r = rn;
  }
  commit_epilogue<T, FEAT>(P, B, c, L, h_rebuild, h_loop, use_cond);
}

// Shared memory of the pipelined kernel per thread: three list heads, two
// own-state pairs and two sets of three partner positions, 16 bytes each,
// then (engines with position remainders) two 8-byte remainders.
constexpr int kAsyncRecords = 3 + 2 * 2 + 2 * 3;
constexpr size_t async_smem(int block, bool prem) {
  return (size_t)kAsyncRecords * block * 16 + (prem ? (size_t)2 * block * 8 : 0);
}

// Software-pipelined grid-stride variant (FP32). A disc's step is two
// dependent gathers deep: its list head, then its partners' positions. Each
// thread keeps three of its discs in flight through shared memory with
// per-thread cp.async copies, so neither gather waits in the iteration that
// needs it: while disc k is computed, the first three partner positions of
// disc k+1, the own state of disc k+1 and the list head of disc k+2 land.
// The copies live in shared memory, not registers, so the depth costs no
// occupancy; each thread reads back only its own copies (no block barrier).
// Layout, 16-byte records indexed [slot][thread]: heads [3], positions [2],
// velocities [2], partner positions [2][3].
//
// WMAJ: the grid's warps take 32-disc chunks warp-major (warp w of CTA b is
// grid warp w * G + b), so that when the chunk count is not a multiple of
// the grid's warps, the warps with one chunk fewer are spread over all CTAs
// instead of filling the last CTAs (which then idle their SMs early).
// PW (engines with bonds): each disc's bond slot words, bond count and strain
// are staged with its own state, one disc ahead, into [2][BMAX][BLOCK] words,
// [2][BLOCK] counts and [2][BLOCK] strains after the records above, so the
// bond partners' gathers start without a dependent load.
template <class T, int MODE, int BLOCK, int MINB, bool FEAT, bool WMAJ = false, bool PW = false>
__global__ void __launch_bounds__(BLOCK, MINB) force_kernel_async(Params<T> P, Bufs<T> B,
                                                                  cudaGraphConditionalHandle h_rebuild,
                                                                  cudaGraphConditionalHandle h_loop, int use_cond,
                                                                  int primed, StepHint hint) {
  static_assert(MODE != kPeek, "read-back uses force_kernel");
  static_assert(sizeof(V4<T>) == 16, "one 16-byte copy per record");
  using bulk::cp16;
  using bulk::cp8;
  using bulk::cp_commit;
  using bulk::cp_wait;
  extern __shared__ uint4 async_smem_base[];
  const StepCtl c = load_step_ctl(B.ctl, hint);
  const int sp = c.sp, lp = c.lp;
  const int t = threadIdx.x;
  const int end = P.n;
  const int stride = gridDim.x * BLOCK;
  uint4* sh = async_smem_base;                                           // [3][BLOCK]
  V4<T>* spos = reinterpret_cast<V4<T>*>(async_smem_base + 3 * BLOCK);  // [2][BLOCK]
  V4<T>* svel = spos + 2 * BLOCK;                                        // [2][BLOCK]
  V4<T>* sq = svel + 2 * BLOCK;                                          // [2][3][BLOCK]
  float2* srem = reinterpret_cast<float2*>(sq + 6 * BLOCK);              // [2][BLOCK]
  const bool pr = P.prem != 0;
  const float2* __restrict__ prem = B.prem[lp];
  const V4<T>* __restrict__ pos = B.pos[sp];
  const V4<T>* __restrict__ vel = B.vel[sp];
  const uint4* __restrict__ head = B.head[lp];
  const GlobalFetch<T> fetch{pos, vel};
  ThreadLedger<T> L;
  // bond staging (PW): slot words, counts and strains of the disc in flight
  const int BM = (PW && FEAT) ? P.BMAX : 0;
  unsigned* sbw = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned char*>(async_smem_base) +
                                              (size_t)kAsyncRecords * BLOCK * 16 + (pr ? (size_t)2 * BLOCK * 8 : 0));
  int* sbc = reinterpret_cast<int*>(sbw + 2 * BM * BLOCK);
  T* ssi = reinterpret_cast<T*>(sbc + 2 * BLOCK);
  auto stage_bonds = [&](int d, int s) {
    if (BM > 0) {
      for (int u = 0; u < BM; ++u) bulk::cp4(sbw + (s * BM + u) * BLOCK + t, B.bpart[lp] + (size_t)u * end + d);
      bulk::cp4(sbc + s * BLOCK + t, B.bcnt[lp] + d);
      bulk::cp4(ssi + s * BLOCK + t, B.strain + d);
      // the warp's 32 discs' reference vectors, histories and strengths
      // towards L2 (one row segment of one slot array per lane; whole warps
      // only, each range rounded inwards to 16-byte bounds)
      const int lane = t & 31, base = d - lane;
      if (WMAJ && base + 32 <= end && lane < 3 * BM) {
        const int u = lane / 3, a = lane - 3 * u;
        const size_t k = (size_t)u * end + base;
        const char* lo = a == 0   ? reinterpret_cast<const char*>(B.bref[lp] + k)
                         : a == 1 ? reinterpret_cast<const char*>(B.bus[lp] + k)
                                  : reinterpret_cast<const char*>(B.bstr[lp] + k);
        const char* hi = lo + 32 * (a == 2 ? sizeof(T) : sizeof(V2<T>));
        const uintptr_t l16 = ((uintptr_t)lo + 15) & ~(uintptr_t)15, h16 = (uintptr_t)hi & ~(uintptr_t)15;
        if (h16 > l16) bulk::prefetch_l2(reinterpret_cast<const void*>(l16), (unsigned)(h16 - l16));
      }
    }
  };
  // partner positions of the disc whose head sits in head slot h, into set s
  auto gather = [&](int h, int s) {
    const uint4 hd = sh[h * BLOCK + t];
    const int cnt = (int)(hd.x & 0xFFu);
    V4<T>* q = sq + (size_t)s * 3 * BLOCK + t;
    if (cnt > 0) cp16(q, pos + hd.y);
    if (cnt > 1) cp16(q + BLOCK, pos + hd.z);
    if (cnt > 2) cp16(q + 2 * BLOCK, pos + hd.w);
  };
  int i = WMAJ ? (int)(((t >> 5) * gridDim.x + blockIdx.x) * 32 + (t & 31)) : (int)(blockIdx.x * BLOCK + t);
  // prologue: heads of the first two discs and the first disc's own state,
  // then the first disc's partners
  if (i < end) {
    cp16(sh + t, head + i);
    cp16(spos + t, pos + i);
    cp16(svel + t, vel + i);
    if (pr) cp8(srem + t, prem + i);
    stage_bonds(i, 0);
  }
  if (i + stride < end) cp16(sh + BLOCK + t, head + i + stride);
  cp_commit();
  cp_wait<0>();
  if (i < end) gather(0, 0);
  cp_commit();
  int h0 = 0;  // head slot of disc k; disc k+1 uses h0+1, disc k+2 h0+2 (mod 3)
  int s = 0;   // own-state and partner set of disc k; disc k+1 uses s^1
  for (; i < end; i += stride) {
    const int h1 = h0 == 2 ? 0 : h0 + 1, h2 = h1 == 2 ? 0 : h1 + 1;
    const int i1 = i + stride, i2 = i1 + stride;
    // group X_k: head of disc k+2, own state of disc k+1
    if (i2 < end) cp16(sh + h2 * BLOCK + t, head + i2);
    if (i1 < end) {
      cp16(spos + (s ^ 1) * BLOCK + t, pos + i1);
      cp16(svel + (s ^ 1) * BLOCK + t, vel + i1);
      if (pr) cp8(srem + (s ^ 1) * BLOCK + t, prem + i1);
      stage_bonds(i1, s ^ 1);
    }
    cp_commit();
    cp_wait<2>();  // X_{k-1} landed: the head of disc k+1
    // group Y_k: partners of disc k+1
    if (i1 < end) gather(h1, s ^ 1);
    cp_commit();
    cp_wait<2>();  // Y_{k-1} landed: the partners of disc k
    const uint4 hd = sh[h0 * BLOCK + t];
    const V4<T> p = spos[s * BLOCK + t];
    const V4<T> v = svel[s * BLOCK + t];
    const V4<T>* q = sq + (size_t)s * 3 * BLOCK + t;
    const int cnt = (int)(hd.x & 0xFFu);
    V4<T> q0{}, q1{}, q2{};
    if (cnt > 0) q0 = q[0];
    if (cnt > 1) q1 = q[BLOCK];
    if (cnt > 2) q2 = q[2 * BLOCK];
    const float2 rm = pr ? srem[s * BLOCK + t] : make_float2(0.0f, 0.0f);
    if constexpr (PW && FEAT) {
      process_particle_q<T, MODE, FEAT, GlobalFetch<T>, false, true>(
          P, B, fetch, sp, lp, i, p, v, hd, q0, q1, q2, primed, c.evals, L, &rm, sbw + s * BM * BLOCK + t, BLOCK,
          BM > 0 ? sbc[s * BLOCK + t] : 0, BM > 0 ? ssi[s * BLOCK + t] : T(0));
    } else {
      process_particle_q<T, MODE, FEAT>(P, B, fetch, sp, lp, i, p, v, hd, q0, q1, q2, primed, c.evals, L, &rm);
    }
    h0 = h1;
    s ^= 1;
  }
  cp_wait<0>();
  commit_epilogue<T, FEAT>(P, B, c, L, h_rebuild, h_loop, use_cond);
}

// Shared memory of the bond staging of a PW pipelined kernel.
inline size_t async_bond_smem(int block, int bmax) { return (size_t)2 * block * ((size_t)bmax * 4 + 4 + 4); }

// Neighbour-window variant (FP32). Each CTA (one per SM) owns a contiguous
// range of sorted particles and walks it two ring blocks (2 x 256 particles)
// per iteration. Positions and velocities of a sliding window of sorted
// indices, the iteration's blocks plus kWinHalo blocks on either side, sit in
// a shared-memory ring of kWinSlots blocks; one thread streams blocks in ahead
// of use with cp.async.bulk (each completing on its own mbarrier, up to
// kWinAhead blocks past the window), and the list heads of the CTA's own
// blocks likewise into a ring of kWinHeads blocks. After the Morton sort a
// disc's partners are nearby in index, so partner gathers read shared memory;
// the few partners outside the window (across a tile row of the cell key)
// read HBM. Waits are bounded; a CTA whose wait runs out sets kStatusTimeout,
// drains its copies in flight (bounded) and stops.
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s of SM clock per wait
constexpr int kWinBlock = 256;     // particles per ring block
constexpr int kWinSlots = 16;      // ring blocks (4096 particles)
constexpr int kWinHalo = 3;        // halo blocks on either side of an iteration
constexpr int kWinAhead = 6;       // blocks streamed past the window
constexpr int kWinHeads = 8;       // head-ring blocks
constexpr int kWinThreads = 2 * kWinBlock;
constexpr size_t kWinSmem = (size_t)kWinSlots * kWinBlock * 2 * sizeof(V4<float>) +
                            (size_t)kWinHeads * kWinBlock * sizeof(uint4) + (kWinSlots + kWinHeads) * 8;

template <class T, int MODE, bool FEAT>
__global__ void __launch_bounds__(kWinThreads, 1) force_kernel_win(Params<T> P, Bufs<T> B,
                                                                   cudaGraphConditionalHandle h_rebuild,
                                                                   cudaGraphConditionalHandle h_loop, int use_cond,
                                                                   int primed, StepHint hint) {
  static_assert(MODE != kPeek && sizeof(T) == 4, "the window variant steps FP32 engines");
  extern __shared__ __align__(128) unsigned char win_smem[];
  V4<T>* spos = reinterpret_cast<V4<T>*>(win_smem);
  V4<T>* svel = spos + kWinSlots * kWinBlock;
  uint4* shead = reinterpret_cast<uint4*>(svel + kWinSlots * kWinBlock);
  uint64_t* bar = reinterpret_cast<uint64_t*>(shead + kWinHeads * kWinBlock);  // [slots] pos/vel, [heads] head
  const StepCtl c = load_step_ctl(B.ctl, hint);
  const int sp = c.sp, lp = c.lp;
  const int n = P.n;
  const int nblk = (n + kWinBlock - 1) / kWinBlock;
  const int b0 = (int)(((long long)blockIdx.x * nblk) / gridDim.x);
  const int b1 = (int)(((long long)(blockIdx.x + 1) * nblk) / gridDim.x);
  const int first = max(0, b0 - kWinHalo);          // first ring block this CTA loads
  const int last = min(nblk - 1, b1 - 1 + kWinHalo);  // last one
  const int tid = threadIdx.x;
  ThreadLedger<T> L;
  if (tid == 0) {
    for (int q = 0; q < kWinSlots + kWinHeads; ++q) bulk::mbar_init(&bar[q], 1);
    bulk::fence_mbar_init();
  }
  __syncthreads();
  int next_pv = first, next_hd = b0;  // next blocks to issue (thread 0)
  auto issue_upto = [&](int k) {      // iteration at blocks k, k + 1
    const int pv_end = min(last, k + 1 + kWinHalo + kWinAhead);
    for (; next_pv <= pv_end; ++next_pv) {
      const int r = next_pv - first, slot = r & (kWinSlots - 1);
      const int cnt = min(kWinBlock, n - next_pv * kWinBlock);
      const uint32_t bytes = (uint32_t)(cnt * sizeof(V4<T>));
      bulk::mbar_arrive_expect_tx(&bar[slot], 2 * bytes);
      bulk::copy_g2s(spos + slot * kWinBlock, B.pos[sp] + (size_t)next_pv * kWinBlock, bytes, &bar[slot]);
      bulk::copy_g2s(svel + slot * kWinBlock, B.vel[sp] + (size_t)next_pv * kWinBlock, bytes, &bar[slot]);
    }
    const int hd_end = min(b1 - 1, k + kWinHeads - 1);
    for (; next_hd <= hd_end; ++next_hd) {
      const int r = next_hd - b0, slot = r & (kWinHeads - 1);
      const int cnt = min(kWinBlock, n - next_hd * kWinBlock);
      const uint32_t bytes = (uint32_t)(cnt * sizeof(uint4));
      bulk::mbar_arrive_expect_tx(&bar[kWinSlots + slot], bytes);
      bulk::copy_g2s(shead + slot * kWinBlock, B.head[lp] + (size_t)next_hd * kWinBlock, bytes,
                     &bar[kWinSlots + slot]);
    }
  };
  if (tid == 0 && b0 < b1) issue_upto(b0);
  int waited_pv = first - 1;  // highest ring block this thread has seen complete
  int waited_hd = b0 - 1;     // highest head block this thread has seen complete
  bool ok = true, failed = false;
  for (int k = b0; k < b1; k += 2) {
    // the window's new blocks and this iteration's heads
    const int need = min(last, k + 1 + kWinHalo);
    while (ok && waited_pv < need) {
      const int r = waited_pv + 1 - first;
      ok = bulk::mbar_wait_bounded(&bar[r & (kWinSlots - 1)], (uint32_t)((r >> 4) & 1), P.wait_budget);
      if (ok) ++waited_pv;
    }
    while (ok && waited_hd < min(k + 1, b1 - 1)) {
      const int r = waited_hd + 1 - b0;
      ok = bulk::mbar_wait_bounded(&bar[kWinSlots + (r & (kWinHeads - 1))], (uint32_t)((r >> 3) & 1),
                                   P.wait_budget);
      if (ok) ++waited_hd;
    }
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const int blk = k + (tid >= kWinBlock ? 1 : 0);
    const int i = blk * kWinBlock + (tid & (kWinBlock - 1));
    if (blk < b1 && i < n) {
      const int off = first * kWinBlock;
      // resident: ring blocks max(first, k - halo) .. min(last, k + 1 + halo)
      const WindowFetch<T> fetch{B.pos[sp], B.vel[sp], spos, svel, max(first, k - kWinHalo) * kWinBlock,
                                 min(n, min(last + 1, k + 2 + kWinHalo) * kWinBlock), off,
                                 kWinSlots * kWinBlock - 1};
      const V4<T> p = spos[(i - off) & fetch.mask];
      const V4<T> v = svel[(i - off) & fetch.mask];
      const uint4 hd = shead[((blk - b0) & (kWinHeads - 1)) * kWinBlock + (tid & (kWinBlock - 1))];
      V4<T> q0{}, q1{}, q2{};
      load_head_partners<T>(fetch, hd, q0, q1, q2);
      process_particle_q<T, MODE, FEAT>(P, B, fetch, sp, lp, i, p, v, hd, q0, q1, q2, primed, c.evals, L);
    }
    __syncthreads();  // every thread is done with the slots the next copies overwrite
    if (tid == 0) issue_upto(k + 2);
  }
  if (failed) {
    if (tid == 0) {
      atomicOr(&B.ctl->status, (int)kStatusTimeout);
      // drain the copies in flight before the CTA's shared memory is released
      for (int b = waited_pv + 1; b < next_pv; ++b) {
        const int r = b - first;
        bulk::mbar_wait_bounded(&bar[r & (kWinSlots - 1)], (uint32_t)((r >> 4) & 1), kWaitBudget);
      }
      for (int b = waited_hd + 1; b < next_hd; ++b) {
        const int r = b - b0;
        bulk::mbar_wait_bounded(&bar[kWinSlots + (r & (kWinHeads - 1))], (uint32_t)((r >> 3) & 1), kWaitBudget);
      }
    }
    __syncthreads();
  }
  commit_epilogue<T, FEAT>(P, B, c, L, h_rebuild, h_loop, use_cond);
}

// Bulk-copy variant: each block streams its tiles of own-particle state
// (position, velocity, list head: 48 B per particle in FP32) from HBM into
// shared memory with cp.async.bulk, double-buffered on two mbarriers, so the
// next tile is in flight while the current one is computed. Partner state is
// gathered from global memory (mostly L2 hits thanks to the cell sort).
template <class T, int MODE, int BLOCK, int MINB, bool FEAT>
__global__ void __launch_bounds__(BLOCK, MINB) force_kernel_bulk(Params<T> P, Bufs<T> B,
                                                                 cudaGraphConditionalHandle h_rebuild,
                                                                 cudaGraphConditionalHandle h_loop, int use_cond,
                                                                 int primed, StepHint hint) {
  static_assert(MODE != kPeek, "read-back uses force_kernel");
  __shared__ alignas(128) V4<T> s_pos[2][BLOCK];
  __shared__ alignas(128) V4<T> s_vel[2][BLOCK];
  __shared__ alignas(128) uint4 s_head[2][BLOCK];
  __shared__ alignas(8) uint64_t s_bar[2];
  const StepCtl c = load_step_ctl(B.ctl, hint);
  const int sp = c.sp, lp = c.lp;
  const long long eval = c.evals;
  const int n = P.n;
  const int ntiles = (n + BLOCK - 1) / BLOCK;
  ThreadLedger<T> L;
  if (threadIdx.x == 0) {
    bulk::mbar_init(&s_bar[0], 1);
    bulk::mbar_init(&s_bar[1], 1);
    bulk::fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int tile, int buf) {
    const int start = tile * BLOCK;
    const int cnt = min(BLOCK, n - start);
    const uint32_t vb = (uint32_t)(cnt * sizeof(V4<T>));
    const uint32_t hb = (uint32_t)(cnt * sizeof(uint4));
    bulk::mbar_arrive_expect_tx(&s_bar[buf], 2 * vb + hb);
    bulk::copy_g2s(&s_pos[buf][0], B.pos[sp] + start, vb, &s_bar[buf]);
    bulk::copy_g2s(&s_vel[buf][0], B.vel[sp] + start, vb, &s_bar[buf]);
    bulk::copy_g2s(&s_head[buf][0], B.head[lp] + start, hb, &s_bar[buf]);
  };
  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles) issue(tile, 0);
  for (int k = 0; tile < ntiles; tile += gridDim.x, ++k) {
    const int buf = k & 1;
    const int next = tile + gridDim.x;
    // buf ^ 1 was released by the barrier that ended the previous iteration
    if (threadIdx.x == 0 && next < ntiles) issue(next, buf ^ 1);
    const bool ok = bulk::mbar_wait_bounded(&s_bar[buf], (uint32_t)((k >> 1) & 1), P.wait_budget);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(&B.ctl->status, (int)kStatusTimeout);
        // let the copies in flight land before the block's shared memory goes
        bulk::mbar_wait_bounded(&s_bar[buf], (uint32_t)((k >> 1) & 1), kWaitBudget);
        if (next < ntiles) bulk::mbar_wait_bounded(&s_bar[buf ^ 1], (uint32_t)(((k + 1) >> 1) & 1), kWaitBudget);
      }
      __syncthreads();
      break;
    }
    const int i = tile * BLOCK + threadIdx.x;
    if (i < n) {
      const V4<T> p = s_pos[buf][threadIdx.x];
      const V4<T> v = s_vel[buf][threadIdx.x];
      const uint4 hd = s_head[buf][threadIdx.x];
      process_particle<T, MODE, FEAT>(P, B, sp, lp, i, p, v, hd, primed, eval, L);
    }
    __syncthreads();
  }
  commit_epilogue<T, FEAT>(P, B, c, L, h_rebuild, h_loop, use_cond);
}

// ---------------------------------------------------------------------------
// Rebuild pipeline. Every kernel is a no-op unless ctl->rebuild_pending.
// ---------------------------------------------------------------------------

// 1. new integer cell and offset of every particle; count per key.
// MULTI: the instance's own grid and key range; particles of a retired
// instance, or of one that went non-finite during a step, take the dead key
// (ctl->key_hi) and fall off the end of the sorted arrays.
template <class T, bool MULTI = false>
__global__ void bin_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int sp = ctl->sp, lp = ctl->lp;
  const int n = MULTI ? ctl->n_old : P.n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int inst = 0;
    if (MULTI) {
      inst = B.inst[lp][i];
      const int st = B.istate[inst];
      if (!(st & kInstAlive) || (st & kStatusNonfinite)) {
        B.tmp_key[i] = ctl->key_hi;
        atomicAdd(&B.cell_count[ctl->key_hi], 1);
        continue;
      }
    }
    const Params<T>& Q = MULTI ? B.iparams[inst] : P;
    const V4<T> p = B.pos[sp][i];
    const int c = lane_to_cell(p.w);
    const int cx = c & 0xFFFF, cy = c >> 16;
    T ox = p.x, oy = p.y;
    int status = 0;
    if (!(isfinite(ox) && isfinite(oy))) {
      status |= kStatusNonfinite;
      ox = T(0);
      oy = T(0);
    }
    const T fx = floor(ox * Q.inv_cell), fy = floor(oy * Q.inv_cell);
    // clamp the shift so that a runaway particle cannot overflow the int maths
    const int kx = (int)fmin(fmax(fx, T(-65536)), T(65536));
    const int ky = (int)fmin(fmax(fy, T(-65536)), T(65536));
    const int nx = cx + kx, ny = cy + ky;
    const int cxn = min(max(nx, 0), Q.ncx - 1), cyn = min(max(ny, 0), Q.ncy - 1);
    if (nx < -1 || nx > Q.ncx || ny < -1 || ny > Q.ncy) status |= kStatusEscaped;
    const int sx = cxn - cx, sy = cyn - cy;
    const T nox = fma((T)(-sx), Q.cell, ox);
    const T noy = fma((T)(-sy), Q.cell, oy);
    B.tmp_cell[i] = cxn | (cyn << 16);
    B.tmp_off[i] = V2<T>{nox, noy};
    // MULTI: what the rebuild finds goes to bits kInstRebuildShift.. of the
    // instance word, so that it cannot change this rebuild's dead/live split
    if (status) atomicOr(MULTI ? &B.istate[inst] : &ctl->status, MULTI ? (status << kInstRebuildShift) : status);
    const int key = MULTI ? Q.key_off + cyn * Q.ncx + cxn : tile_key(cxn, cyn, P.tiles_x);
    if (MULTI) B.tmp_key[i] = key;
    atomicAdd(&B.cell_count[key], 1);
  }
}

// 2. exclusive scan of the per-key counts (three phases, 4096 keys per block).
// n < 0: the batched engine's key count, ctl->key_hi + 1 (dead key included).
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  __shared__ int warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    warp_sums[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const int before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__device__ __forceinline__ int scan_count(const Ctl* ctl, int n) { return n >= 0 ? n : ctl->key_hi + 1; }

static __global__ void scan_blocks_kernel(const Ctl* ctl, const int* in, int* out, int* block_sums, int n_arg) {
  if (!ctl->rebuild_pending) return;
  const int n = scan_count(ctl, n_arg);
  if (blockIdx.x * kScanChunk >= n) return;  // whole block out of range (uniform)
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
  int v[kScanItems];
  int local = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    local += v[k];
  }
  int total;
  int run = block_exclusive_scan(local, &total);
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// One block; any number of block sums, kScanChunk at a time with a carry.
static __global__ void scan_top_kernel(const Ctl* ctl, int* block_sums, int n_arg) {
  if (!ctl->rebuild_pending) return;
  const int nblocks = (scan_count(ctl, n_arg) + kScanChunk - 1) / kScanChunk;
  int carry = 0;
  for (int c0 = 0; c0 < nblocks; c0 += kScanChunk) {
    const int base = c0 + threadIdx.x * kScanItems;
    int v[kScanItems];
    int local = 0;
    for (int k = 0; k < kScanItems; ++k) {
      v[k] = (base + k < nblocks) ? block_sums[base + k] : 0;
      local += v[k];
    }
    int total;
    int run = carry + block_exclusive_scan(local, &total);
    for (int k = 0; k < kScanItems; ++k) {
      if (base + k < nblocks) block_sums[base + k] = run;
      run += v[k];
    }
    carry += total;
  }
}

static __global__ void scan_add_kernel(const Ctl* ctl, int* out, const int* block_sums, int n_arg) {
  if (!ctl->rebuild_pending) return;
  const int n = scan_count(ctl, n_arg);
  const int base = blockIdx.x * kScanChunk;
  if (base >= n) return;
  const int add = block_sums[blockIdx.x];
  for (int k = threadIdx.x; k < kScanChunk; k += blockDim.x)
    if (base + k < n) out[base + k] += add;
}

// 3. scatter old indices into their key's range (order fixed by step 4)
template <class T, bool MULTI = false>
__global__ void scatter_kernel(Params<T> P, Bufs<T> B) {
  const Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int n = MULTI ? ctl->n_old : P.n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int key;
    if (MULTI) {
      key = B.tmp_key[i];
    } else {
      const int c = B.tmp_cell[i];
      key = tile_key(c & 0xFFFF, c >> 16, P.tiles_x);
    }
    const int slot = B.cell_start[key] + atomicAdd(&B.cell_fill[key], 1);
    B.perm[slot] = i;
  }
}

// 4. deterministic order inside each cell: ascending original id (the
// instance-local id in the batched engine; a cell never mixes instances).
// The dead key is left unsorted.
template <class T, bool MULTI = false>
__global__ void cellsort_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int nkeys = MULTI ? ctl->key_hi : P.nkeys;
  const int* orig = B.orig[ctl->lp];
  for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < nkeys; key += gridDim.x * blockDim.x) {
    const int cnt = B.cell_count[key];
    if (cnt < 2) continue;
    const int start = B.cell_start[key];
    for (int a = start + 1; a < start + cnt; ++a) {
      const int x = B.perm[a];
      const int ox = orig[x];
      int b = a - 1;
      while (b >= start && orig[B.perm[b]] > ox) {
        B.perm[b + 1] = B.perm[b];
        --b;
      }
      B.perm[b + 1] = x;
    }
  }
}

// 5. gather particle state into the new order (other buffers)
template <class T, bool MULTI = false>
__global__ void gather_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int sp = ctl->sp, lp = ctl->lp;
  const int nn = MULTI ? ctl->n_live : P.n;  // MULTI: the live count after this rebuild
  const size_t n = (size_t)P.n;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nn; p += gridDim.x * blockDim.x) {
    const int i = B.perm[p];
    const V4<T> q = B.pos[sp][i];
    V2<T> off = B.tmp_off[i];
    if (sizeof(T) == 4 && P.prem) {
      // the offset relative to the new cell, with its remainder carried over:
      // (x, r) + (old cell - new cell) * cell
      const int co = lane_to_cell(q.w), cn = B.tmp_cell[i];
      const float cl = (float)(MULTI ? B.iparams[B.inst[lp][i]].cell : P.cell);
      float2 r = B.prem[lp][i];
      off.x = (T)add_prod_comp((float)q.x, r.x, (float)((co & 0xFFFF) - (cn & 0xFFFF)), cl);
      off.y = (T)add_prod_comp((float)q.y, r.y, (float)((co >> 16) - (cn >> 16)), cl);
      B.prem[lp ^ 1][p] = r;
    }
    B.pos[sp ^ 1][p] = V4<T>{off.x, off.y, q.z, cell_to_lane(B.tmp_cell[i], T(0))};
    B.vel[sp ^ 1][p] = B.vel[sp][i];
    B.orig[lp ^ 1][p] = B.orig[lp][i];
    if (MULTI) B.inst[lp ^ 1][p] = B.inst[lp][i];
    B.invperm[i] = p;
    for (int w = 0; w < 4; ++w) B.whist[lp ^ 1][w * n + p] = B.whist[lp][w * n + i];
  }
}

// 5b. bond slots follow their disc; partners are renamed to the new order
template <class T, bool MULTI = false>
__global__ void bond_gather_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending || P.BMAX == 0) return;
  const int lp = ctl->lp;
  const int nn = MULTI ? ctl->n_live : P.n;
  const size_t n = (size_t)P.n;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nn; p += gridDim.x * blockDim.x) {
    const int i = B.perm[p];
    const int bc = B.bcnt[lp][i];
    B.bcnt[lp ^ 1][p] = bc;
    B.bpinv[lp ^ 1][p] = B.bpinv[lp][i];
    for (int s = 0; s < bc; ++s) {
      const size_t ko = (size_t)s * n + i, kn = (size_t)s * n + p;
      const unsigned w = B.bpart[lp][ko];
      const int jo = (int)(w & kBondIdx);
      const int jn = B.invperm[jo];
      B.bpart[lp ^ 1][kn] = (w & ~kBondIdx) | (unsigned)jn;
      B.bref[lp ^ 1][kn] = B.bref[lp][ko];
      B.bstr[lp ^ 1][kn] = B.bstr[lp][ko];
      // the shear displacement is kept in the orientation of the pair's lower
      // sorted index: flip it when the re-sort swapped the pair's sides
      const V2<T> u = B.bus[lp][ko];
      B.bus[lp ^ 1][kn] = ((i < jo) != (p < jn)) ? V2<T>{-u.x, -u.y} : u;
      B.bfail[lp ^ 1][kn] = B.bfail[lp][ko];
    }
  }
}

// 6. candidate partners: the 3x3 cells around each particle, fixed order
template <class T, bool MULTI = false>
__global__ void build_nbr_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int sp1 = ctl->sp ^ 1, lp1 = ctl->lp ^ 1;
  const int nn = MULTI ? ctl->n_live : P.n;
  const V4<T>* pos = B.pos[sp1];
  unsigned* tail = B.nbr[lp1];
  const size_t n = (size_t)P.n;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nn; p += gridDim.x * blockDim.x) {
    const int inst = MULTI ? B.inst[lp1][p] : 0;
    const Params<T>& Q = MULTI ? B.iparams[inst] : P;
    unsigned first[kHeadSlots] = {0u, 0u, 0u};
    const V4<T> a = pos[p];
    const int c = lane_to_cell(a.w);
    const int cx = c & 0xFFFF, cy = c >> 16;
    // bonded partners are handled through their bond slot (intact or broken)
    const int bc = P.BMAX > 0 ? B.bcnt[lp1][p] : 0;
    int cnt = 0;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= Q.ncy) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        const int x = cx + dx;
        if (x < 0 || x >= Q.ncx) continue;
        const int key = MULTI ? Q.key_off + y * Q.ncx + x : tile_key(x, y, P.tiles_x);
        const int start = B.cell_start[key];
        const int num = B.cell_count[key];
        for (int q = start; q < start + num; ++q) {
          if (q == p) continue;
          bool bonded = false;
          for (int t = 0; t < bc; ++t)
            if ((int)(B.bpart[lp1][(size_t)t * n + p] & kBondIdx) == q) bonded = true;
          if (bonded) continue;
          const V4<T> b = pos[q];
          const T ddx = fma((T)dx, Q.cell, b.x - a.x);
          const T ddy = fma((T)dy, Q.cell, b.y - a.y);
          const T reach = (a.z + b.z) + Q.skin;
          if (ddx * ddx + ddy * ddy <= reach * reach) {
            if (cnt < kHeadSlots)
              first[cnt] = (unsigned)q;
            else if (cnt < P.W)
              tail[(size_t)(cnt - kHeadSlots) * n + p] = (unsigned)q;
            ++cnt;
          }
        }
      }
    }
    if (cnt > P.W) {
      atomicOr(MULTI ? &B.istate[inst] : &ctl->status, (int)kStatusCapacity);
      cnt = P.W;
    }
    B.head[lp1][p] = make_uint4((unsigned)cnt, first[0], first[1], first[2]);
    atomicMax(&ctl->max_cnt, cnt);
  }
}

// 7. tangential-history remap keyed by the original-id pair: each particle
// looks its new partner up in its own old list (old sorted indices through
// perm) and carries the stored displacement over, flipping its sign when the
// pair's lower sorted index changed sides.
template <class T, bool MULTI = false>
__global__ void link_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int lp = ctl->lp;
  const int nn = MULTI ? ctl->n_live : P.n;
  const size_t n = (size_t)P.n;
  const unsigned* nbr = B.nbr[lp ^ 1];
  const unsigned* onbr = B.nbr[lp];
  const V2<T>* ohist = B.hist[lp];
  V2<T>* nhist = B.hist[lp ^ 1];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nn; p += gridDim.x * blockDim.x) {
    const uint4 head = B.head[lp ^ 1][p];
    const int c = (int)(head.x & 0xFFu);
    const int op = B.perm[p];
    const uint4 ohead = B.head[lp][op];
    const int oc = (int)(ohead.x & 0xFFu);
    const unsigned omask = ohead.x >> 8;
    unsigned mask = 0u;
    if (omask) {
      for (int s = 0; s < c; ++s) {
        const int q = slot_partner(head, nbr, n, p, s);
        const int oq = B.perm[q];
        for (int t = 0; t < oc; ++t) {
          if (slot_partner(ohead, onbr, n, op, t) != oq) continue;
          if ((omask >> t) & 1u) {
            V2<T> xi = ohist[(size_t)t * n + op];
            if ((op < oq) != (p < q)) xi = V2<T>{-xi.x, -xi.y};
            nhist[(size_t)s * n + p] = xi;
            mask |= 1u << s;
          }
          break;
        }
      }
    }
    B.head[lp ^ 1][p].x = head.x | (mask << 8);
  }
}

// 8. clear the key counters for the next rebuild
template <class T, bool MULTI = false>
__global__ void clear_keys_kernel(Params<T> P, Bufs<T> B) {
  if (!B.ctl->rebuild_pending) return;
  const int nkeys = MULTI ? B.ctl->key_hi + 1 : P.nkeys;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nkeys; k += gridDim.x * blockDim.x) {
    B.cell_count[k] = 0;
    B.cell_fill[k] = 0;
  }
}

// 9. swap to the new buffers
static __global__ void rebuild_flip_kernel(Ctl* ctl) {
  if (!ctl->rebuild_pending) return;
  ctl->sp ^= 1;
  ctl->lp ^= 1;
  ctl->disp = 0.0f;
  ctl->since = 0;
  ctl->rebuilds += 1;
  ctl->rebuild_pending = 0;
}

// ---------------------------------------------------------------------------
// Host <-> device state conversion (original particle order, FP64)
// ---------------------------------------------------------------------------
template <class T>
__global__ void pack_kernel(Params<T> P, Bufs<T> B, const double* pos, const double* vel, const double* omega,
                            const double* radius, const double* mass, const double* inertia) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  Ctl* ctl = B.ctl;
  const int sp = ctl->sp, lp = ctl->lp;
  const double c = (double)P.cell;
  const double x = pos[2 * i], y = pos[2 * i + 1];
  double fx = floor(x / c), fy = floor(y / c);
  if (!(fx == fx)) fx = 0.0;
  if (!(fy == fy)) fy = 0.0;
  const int cx = (int)fmin(fmax(fx, 0.0), (double)(P.ncx - 1));
  const int cy = (int)fmin(fmax(fy, 0.0), (double)(P.ncy - 1));
  const double r = radius[i], m = mass[i];
  const bool clamped = isinf(m) && m > 0.0;  // infinite mass: a clamped disc
  const double ox = x - cx * c, oy = y - cy * c;
  B.pos[sp][i] = V4<T>{(T)ox, (T)oy, (T)r, cell_to_lane(cx | (cy << 16), T(0))};
  if (sizeof(T) == 4 && P.prem)
    B.prem[lp][i] = make_float2((float)(ox - (double)(T)ox), (float)(oy - (double)(T)oy));
  B.vel[sp][i] = clamped ? V4<T>{T(0), T(0), T(0), T(0)}
                         : V4<T>{(T)vel[2 * i], (T)vel[2 * i + 1], (T)omega[i], (T)(1.0 / m)};
  if (B.bcnt[lp]) B.bcnt[lp][i] = 0;
  B.head[lp][i] = make_uint4(0u, 0u, 0u, 0u);
  B.orig[lp][i] = i;
  for (int w = 0; w < 4; ++w) B.whist[lp][(size_t)w * P.n + i] = V2<T>{T(0), T(0)};
  // the engine models I = kappa m r^2 with one kappa
  const double want = m * r * r / (double)P.kinv;
  if (!clamped && !(fabs(inertia[i] - want) <= 1e-6 * fabs(want))) atomicOr(&ctl->status, (int)kStatusInertia);
}

template <class T>
__global__ void unpack_kernel(Params<T> P, Bufs<T> B, double* pos, double* vel, double* omega, double* force,
                              double* torque) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const Ctl* ctl = B.ctl;
  const int sp = ctl->sp, lp = ctl->lp;
  const int o = B.orig[lp][p];
  const V4<T> q = B.pos[sp][p];
  const int c = lane_to_cell(q.w);
  const double cl = (double)P.cell;
  if (pos) {
    const float2 r = (sizeof(T) == 4 && P.prem) ? B.prem[lp][p] : make_float2(0.0f, 0.0f);
    pos[2 * o] = (double)(c & 0xFFFF) * cl + (double)q.x + (double)r.x;
    pos[2 * o + 1] = (double)(c >> 16) * cl + (double)q.y + (double)r.y;
  }
  const V4<T> v = B.peek_vel[p];
  if (vel) {
    vel[2 * o] = (double)v.x;
    vel[2 * o + 1] = (double)v.y;
  }
  if (omega) omega[o] = (double)v.z;
  const V4<T> f = B.peek_force[p];
  if (force) {
    force[2 * o] = (double)f.x;
    force[2 * o + 1] = (double)f.y;
  }
  if (torque) torque[o] = (double)f.z;
}

static __global__ void set_target_kernel(Ctl* ctl, long long n) { ctl->target = ctl->evals + n; }

static __global__ void request_rebuild_kernel(Ctl* ctl) { ctl->rebuild_pending = 1; }

// Stored tangential history of every pair with a non-zero value, keyed by the
// original ids (lo, hi) and oriented as the displacement of lo relative to hi
// (read from the copy of the pair's lower sorted index).
template <class T>
__global__ void history_kernel(Params<T> P, Bufs<T> B, int* pairs, double* xi, long long capacity,
                               unsigned long long* count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int lp = B.ctl->lp;
  const uint4 head = B.head[lp][p];
  const int c = (int)(head.x & 0xFFu);
  const unsigned mask = head.x >> 8;
  for (int s = 0; s < c; ++s) {
    const int q = slot_partner(head, B.nbr[lp], (size_t)P.n, p, s);
    if (p >= q || !((mask >> s) & 1u)) continue;
    const V2<T> h = B.hist[lp][(size_t)s * P.n + p];
    if (h.x == T(0) && h.y == T(0)) continue;
    const unsigned long long k = atomicAdd(count, 1ull);
    if ((long long)k >= capacity) continue;
    const int a = B.orig[lp][p], b = B.orig[lp][q];
    const double sg = (a < b) ? 1.0 : -1.0;
    pairs[2 * k] = min(a, b);
    pairs[2 * k + 1] = max(a, b);
    xi[2 * k] = sg * (double)h.x;
    xi[2 * k + 1] = sg * (double)h.y;
  }
}

// Candidate pairs as original ids (lower sorted index side only), for tests.
template <class T>
__global__ void pairs_kernel(Params<T> P, Bufs<T> B, int* out, long long capacity, unsigned long long* count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int lp = B.ctl->lp;
  const uint4 head = B.head[lp][p];
  const int c = (int)(head.x & 0xFFu);
  for (int s = 0; s < c; ++s) {
    const int q = slot_partner(head, B.nbr[lp], (size_t)P.n, p, s);
    if (p < q) {
      const unsigned long long k = atomicAdd(count, 1ull);
      if ((long long)k < capacity) {
        const int a = B.orig[lp][p], b = B.orig[lp][q];
        out[2 * k] = min(a, b);
        out[2 * k + 1] = max(a, b);
      }
    }
  }
}

// Engine parameters from the public configuration (material constants in
// closed form: E* = E/(2(1-nu^2)), G* = E/(4(2-nu)(1+nu)), Tsuji beta from the
// restitution coefficient).
template <class T>
inline void make_params(const tdem_hm_config& c, int slots, Params<T>& P) {
  P.n = c.n;
  P.W = slots;
  P.ncx = c.ncx;
  P.ncy = c.ncy;
  P.tiles_x = (c.ncx + 31) / 32;
  const int tiles_y = (c.ncy + 31) / 32;
  P.nkeys = P.tiles_x * tiles_y * 1024;
  P.walls = c.walls;
  P.cell = (T)c.cell;
  P.inv_cell = (T)(1.0 / (double)P.cell);
  P.skin = (T)c.skin;
  P.dt = (T)c.dt;
  P.half_dt = (T)(0.5 * c.dt);
  const double estar = c.young / (2.0 * (1.0 - c.poisson * c.poisson));
  const double gstar = c.young / (4.0 * (2.0 - c.poisson) * (1.0 + c.poisson));
  double beta = 0.0;
  if (c.restitution < 1.0) {
    const double le = std::log(c.restitution);
    beta = -le / std::sqrt(le * le + M_PI * M_PI);
  }
  P.estar2 = (T)(2.0 * estar);
  P.gstar8 = (T)(8.0 * gstar);
  P.damp = (T)(2.0 * std::sqrt(5.0 / 6.0) * beta);
  P.mu = (T)c.mu;
  P.mu_wall = (T)c.mu_wall;
  P.gx = (T)c.gravity[0];
  P.gy = (T)c.gravity[1];
  P.kinv = (T)(1.0 / c.inertia_factor);
  P.rebuild_disp = (float)(0.5 * c.skin * 0.98);
  P.BMAX = c.max_bonds;
  P.kn = (T)c.bond_kn;
  P.ks = (T)c.bond_ks;
  P.bzeta = (T)c.bond_damping;
  P.cn_k = (T)(2.0 * c.bond_damping * std::sqrt(c.bond_kn));
  P.cs_k = (T)(2.0 * c.bond_damping * std::sqrt(c.bond_ks));
  P.eps_t = c.breaking_strain;
  P.eps_s = c.shear_breaking_strain;
  P.ind_x0 = c.indenter_center[0];
  P.ind_y0 = c.indenter_center[1];
  P.ind_vx = c.indenter_velocity[0];
  P.ind_vy = c.indenter_velocity[1];
  P.irad = (T)c.indenter_radius;
  P.load_cap = c.indenter_radius > 0.0 ? std::max(c.load_capacity, 0) : 0;
  auto below = [](double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
  };
  auto above = [](double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
  };
  P.eps_t_lo = below(c.breaking_strain);
  P.eps_t_hi = above(c.breaking_strain);
  P.eps_s_lo = below(c.shear_breaking_strain);
  P.eps_s_hi = above(c.shear_breaking_strain);
  P.ind_x0f = (float)c.indenter_center[0];
  P.ind_y0f = (float)c.indenter_center[1];
  P.ind_dxf = (float)((double)P.dt * c.indenter_velocity[0]);
  P.ind_dyf = (float)((double)P.dt * c.indenter_velocity[1]);
  P.wait_budget = kWaitBudget;
}

}  // namespace hm
}  // namespace tdem
