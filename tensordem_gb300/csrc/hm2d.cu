// Hertz-Mindlin 2-D disc engine on sm_103a: cell-list neighbour build with a
// Verlet skin, history remap across rebuilds, and one fused
// force + velocity-Verlet kernel per step, driven by a conditional CUDA graph
// that decides list rebuilds on the device.
//
// Contact law (per pair a < b in sorted order, n from a to b, delta > 0):
//   F_n = max(2/3 S_n delta + D sqrt(S_n m*) v_n, 0), S_n = 2 E* sqrt(R* delta)
//   xi  = proj_t(xi + v_t dt), |S_t xi| <= mu F_n,    S_t = 8 G* sqrt(R* delta)
//   F_a = -F_n n - S_t xi, F_b = -F_a, tau = r (n x F_a)
// following src/tensordem/scale_ceiling/kernel.py:277-336 (normal, dashpot,
// Cundall-Strack cap), src/tensordem/hertz_mindlin.py:94-176 (Mindlin S_t),
// src/tensordem/granular2d/engine.py:458-503 (2-D levers, torques, tangent
// projection) and src/tensordem/contact_tangential.py:356-417 (history reset
// when the contact opens).
//
// Determinism without float atomics: every particle sums its own contacts in
// its list order; each pair is computed by both partners from the same
// canonically ordered operands, so the two halves are exact negatives.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bulk.cuh"
#include "common.h"
#include "hm2d.cuh"

namespace tdem {
namespace hm {

enum Mode { kPrime = 0, kStep = 1, kPeek = 2 };

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

// One active contact (g.d2 < g.rs^2): force on a, torque lever term, history.
template <class T>
__device__ __forceinline__ PairOut<T> pair_force(const Params<T>& P, const Geo<T>& g, const V4<T>& pa,
                                                 const V4<T>& va, const V4<T>& pb, const V4<T>& vb,
                                                 V2<T> xi) {
  PairOut<T> o;
  o.active = true;
  if (!(va.w + vb.w > T(0))) {  // two clamped discs exchange no force
    o.fx = o.fy = o.cr = o.diss = o.un = o.ut = T(0);
    o.xi = V2<T>{T(0), T(0)};
    return o;
  }
  const T d = dev_sqrt(g.d2);
  const T delta = g.rs - d;
  const T nx = g.dx / d, ny = g.dy / d;
  const T reff = pa.z * pb.z / g.rs;
  const T meff = T(1) / (va.w + vb.w);
  const T sq = dev_sqrt(reff * delta);
  const T sn = P.estar2 * sq;
  const T fel = (T(2) / T(3)) * sn * delta;
  const T wsum = va.z * pa.z + vb.z * pb.z;
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
template <class T, bool COMMIT>
__device__ __forceinline__ void wall_contact(const Params<T>& P, T nwx, T nwy, T gap, const V4<T>& p,
                                             const V4<T>& v, V2<T>* slot, Acc<T>& fx, Acc<T>& fy,
                                             Acc<T>& tq, T& diss, T& un, T& ut, bool peek_old_xi) {
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

template <class T>
__device__ __forceinline__ float block_max_f(float x) {
  __shared__ float s[kThreads / 32];
  for (int off = 16; off > 0; off >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, off));
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = x;
  __syncthreads();
  float m = s[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, s[w]);
  __syncthreads();
  return m;
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
// One candidate slot of particle i (partner j at position q): contact test,
// history update in place, force and torque accumulation.
template <class T, int MODE>
__device__ __forceinline__ void do_slot(const Params<T>& P, const V4<T>* __restrict__ vel,
                                        V2<T>* __restrict__ hist, int i, int j, int s, size_t slot,
                                        const V4<T>& p, const V4<T>& v, const V4<T>& q, unsigned mask,
                                        unsigned& nmask, Acc<T>& fx, Acc<T>& fy, Acc<T>& tq, T& diss, T& un,
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
  const V4<T> w = vel[j];
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

// Per-disc objective shear invariant over the disc's initial bonds (broken or
// not), the reference's local Green-Lagrange measure (dem.py:182-208) written
// with G = F - I: E = (G + G^T + G^T G) / 2.
template <class T>
__global__ void strain_kernel(Params<T> P, Bufs<T> B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const int bc = B.bcnt[lp][i];
  T sv = T(0);
  if (bc > 0) {
    const V4<T>* pos = B.pos[sp];
    const V4<T> p = pos[i];
    T g00 = 0, g01 = 0, g10 = 0, g11 = 0;
    for (int s = 0; s < bc; ++s) {
      const size_t k = (size_t)s * P.n + i;
      const int j = (int)(B.bpart[lp][k] & kBondIdx);
      const V2<T> cur = cell_delta<T>(P, p, pos[j]);
      const V2<T> r = B.bref[lp][k];
      const T ux = cur.x - r.x, uy = cur.y - r.y;
      g00 += ux * r.x;
      g01 += ux * r.y;
      g10 += uy * r.x;
      g11 += uy * r.y;
    }
    const V4<T> q = B.bpinv[lp][i];
    const T f00 = g00 * q.x + g01 * q.z, f01 = g00 * q.y + g01 * q.w;
    const T f10 = g10 * q.x + g11 * q.z, f11 = g10 * q.y + g11 * q.w;
    const T e00 = T(0.5) * (T(2) * f00 + f00 * f00 + f10 * f10);
    const T e11 = T(0.5) * (T(2) * f11 + f01 * f01 + f11 * f11);
    const T e01 = T(0.5) * ((f01 + f10) + f00 * f01 + f10 * f11);
    const T dd = e00 - e11;
    sv = dev_sqrt(dd * dd + T(4) * (e01 * e01));
  }
  B.strain[i] = sv;
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

// One bond slot s of disc i: the break test (FP64 comparison of the strains
// against the bond's thresholds), then the bond law while intact, or the Hertz
// contact with the slot's history once broken (dem.py:243-292 semantics: a
// bond broken at this evaluation already acts as a contact).
template <class T, int MODE>
__device__ __forceinline__ void do_bond(const Params<T>& P, const Bufs<T>& B, int sp, int lp, int i, int s,
                                        long long eval, const V4<T>& p, const V4<T>& v, Acc<T>& fx, Acc<T>& fy,
                                        Acc<T>& tq, ThreadLedger<T>& L, int primed) {
  constexpr bool COMMIT = MODE != kPeek;
  const size_t k = (size_t)s * P.n + i;
  const unsigned w = B.bpart[lp][k];
  const int j = (int)(w & kBondIdx);
  const V4<T> q = B.pos[sp][j];
  const V4<T> wv = B.vel[sp][j];
  const bool owner = i < j;
  const V4<T>& a = owner ? p : q;
  const V4<T>& b = owner ? q : p;
  const V4<T>& va = owner ? v : wv;
  const V4<T>& vb = owner ? wv : v;
  const V2<T> rs = B.bref[lp][k];
  const V2<T> ref = owner ? rs : V2<T>{-rs.x, -rs.y};
  const Geo<T> g = pair_geo<T>(P, a, b);
  bool broken = (w & kBondBroken) != 0u;
  V2<T> us = B.bus[lp][k];
  if (!broken) {
    const T ux = g.dx - ref.x, uy = g.dy - ref.y;
    const T d = dev_sqrt(g.d2);
    const T l0 = dev_sqrt(ref.x * ref.x + ref.y * ref.y);
    const T ext = (T(2) * (ref.x * ux + ref.y * uy) + (ux * ux + uy * uy)) / (d + l0);
    const T tensile = ext / l0;
    const T shear = T(0.5) * (B.strain[i] + B.strain[j]);
    const double str = (double)B.bstr[lp][k];
    const bool bt = (double)tensile > P.eps_t * str;
    const bool bs = (double)shear > P.eps_s * str;
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
      const T nx = g.dx / d, ny = g.dy / d;
      const T meff = T(1) / (va.w + vb.w);
      const T wsum = va.z * a.z + vb.z * b.z;
      const T vrx = (va.x - vb.x) - wsum * ny;
      const T vry = (va.y - vb.y) + wsum * nx;
      const T vn = vrx * nx + vry * ny;
      const T vtx = vrx - vn * nx, vty = vry - vn * ny;
      T sx = us.x + vtx * P.dt, sy = us.y + vty * P.dt;
      const T sn = sx * nx + sy * ny;
      sx -= sn * nx;
      sy -= sn * ny;
      const T cn = T(2) * P.bzeta * dev_sqrt(P.kn * meff);
      const T cs = T(2) * P.bzeta * dev_sqrt(P.ks * meff);
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
template <class T>
__device__ __forceinline__ void indenter_contact(const Params<T>& P, long long eval, const V4<T>& p, const V4<T>& v,
                                                 Acc<T>& fx, Acc<T>& fy, ThreadLedger<T>& L) {
  const int c = lane_to_cell(p.w);
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

// Everything one particle does in one evaluation: its candidate slots, the
// walls, and (committing modes) the velocity-Verlet update into the other
// buffers. p, v, hd are the particle's own loads (already issued).
template <class T, int MODE, bool FEAT>
__device__ __forceinline__ void process_particle(const Params<T>& P, const Bufs<T>& B, int sp, int lp, int i,
                                                 const V4<T>& p, const V4<T>& v, const uint4& hd, int primed,
                                                 long long eval, ThreadLedger<T>& L) {
  constexpr bool COMMIT = MODE != kPeek;
  const int n = P.n;
  const V4<T>* __restrict__ pos = B.pos[sp];
  const V4<T>* __restrict__ vel = B.vel[sp];
  const unsigned* __restrict__ tail = B.nbr[lp];
  V2<T>* __restrict__ hist = B.hist[lp];
  const int cnt = (int)(hd.x & 0xFFu);
  const unsigned mask = hd.x >> 8;
  // positions of the first three partners, issued together
  V4<T> q0{}, q1{}, q2{};
  if (cnt > 0) q0 = pos[hd.y];
  if (cnt > 1) q1 = pos[hd.z];
  if (cnt > 2) q2 = pos[hd.w];
  unsigned nmask = 0u;
  Acc<T> fx, fy, tq;
  if (FEAT && P.BMAX > 0) {
    const int bc = B.bcnt[lp][i];
    for (int s = 0; s < bc; ++s) do_bond<T, MODE>(P, B, sp, lp, i, s, eval, p, v, fx, fy, tq, L, primed);
  }
  if (cnt > 0)
    do_slot<T, MODE>(P, vel, hist, i, (int)hd.y, 0, (size_t)i, p, v, q0, mask, nmask, fx, fy, tq, L.diss, L.un,
                     L.ut, primed);
  if (cnt > 1)
    do_slot<T, MODE>(P, vel, hist, i, (int)hd.z, 1, (size_t)n + i, p, v, q1, mask, nmask, fx, fy, tq, L.diss,
                     L.un, L.ut, primed);
  if (cnt > 2)
    do_slot<T, MODE>(P, vel, hist, i, (int)hd.w, 2, (size_t)2 * n + i, p, v, q2, mask, nmask, fx, fy, tq, L.diss,
                     L.un, L.ut, primed);
  for (int s = kHeadSlots; s < cnt; ++s) {
    const int j = (int)tail[(size_t)(s - kHeadSlots) * n + i];
    const V4<T> q = pos[j];
    do_slot<T, MODE>(P, vel, hist, i, j, s, (size_t)s * n + i, p, v, q, mask, nmask, fx, fy, tq, L.diss, L.un,
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
      const double x = (double)(c & 0xFFFF) * (double)P.cell + (double)p.x;
      const double y = (double)(c >> 16) * (double)P.cell + (double)p.y;
      L.pe += -m * ((double)P.gx * x + (double)P.gy * y);
    }
  } else {
    T vx, vy, om;
    if (MODE == kPrime) {
      vx = v.x + P.half_dt * ax;
      vy = v.y + P.half_dt * ay;
      om = v.z + P.half_dt * al;
    } else {
      vx = (v.x + P.half_dt * ax) + P.half_dt * ax;
      vy = (v.y + P.half_dt * ay) + P.half_dt * ay;
      om = (v.z + P.half_dt * al) + P.half_dt * al;
    }
    const T ox = p.x + P.dt * vx;
    const T oy = p.y + P.dt * vy;
    B.pos[sp ^ 1][i] = V4<T>{ox, oy, p.z, p.w};
    B.vel[sp ^ 1][i] = V4<T>{vx, vy, om, v.w};
    L.vmax2 = fmaxf(L.vmax2, (float)(vx * vx + vy * vy));
    if (!(isfinite(ox) && isfinite(oy) && isfinite(vx) && isfinite(vy) && isfinite(om))) L.bad = true;
  }
}

// Commit epilogue: per-warp ledger partials and the speed bound, then the
// last warp of the last block does the step bookkeeping (indenter reaction,
// rebuild trigger) and sets the graph's conditions. No block-wide barrier:
// warps retire as soon as they are done.
template <class T, bool FEAT>
__device__ __forceinline__ void commit_epilogue(const Params<T>& P, const Bufs<T>& B, int sp,
                                                const ThreadLedger<T>& L, cudaGraphConditionalHandle h_rebuild,
                                                cudaGraphConditionalHandle h_loop, int use_cond) {
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
  if (__any_sync(0xffffffffu, L.bad) && (threadIdx.x & 31) == 0) atomicOr(&ctl->status, (int)kStatusNonfinite);
  __shared__ unsigned s_warps_done;
  if (threadIdx.x == 0) s_warps_done = 0u;  // every block starts at zero
  __syncthreads();
  if ((threadIdx.x & 31) != 0) return;
  const size_t gw = (size_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (wd != T(0)) B.diss_part[gw] += (double)wd;
  if (FEAT && wf != T(0)) B.frac_part[gw] += (double)wf;
  if (FEAT && wb) atomicAdd(&ctl->broken, wb);
  if (FEAT && (wix != T(0) || wiy != T(0))) {
    const unsigned e = atomicAdd(&ctl->load_entries, 1u);
    B.ind_part[3 * (size_t)e] = (double)gw;
    B.ind_part[3 * (size_t)e + 1] = (double)wix;
    B.ind_part[3 * (size_t)e + 2] = (double)wiy;
  }
  const unsigned bits = __float_as_uint(wm);
  if (bits > *reinterpret_cast<volatile unsigned*>(&ctl->vmax2_bits)) atomicMax(&ctl->vmax2_bits, bits);
  __threadfence();
  const unsigned mine = atomicAdd(&s_warps_done, 1u);
  if (mine != blockDim.x / 32 - 1) return;
  // last warp of this block
  const unsigned t = atomicAdd(&ctl->ticket, 1u);
  if (t != gridDim.x - 1) return;
  // last block of the grid
  __threadfence();
  if (FEAT && P.irad > T(0)) {
    // sum the indenter partials in warp order (deterministic)
    const unsigned m = *reinterpret_cast<volatile unsigned*>(&ctl->load_entries);
    double* e = B.ind_part;
    for (unsigned a = 1; a < m; ++a) {
      const double k0 = e[3 * a], k1 = e[3 * a + 1], k2 = e[3 * a + 2];
      unsigned b = a;
      while (b > 0 && e[3 * (b - 1)] > k0) {
        e[3 * b] = e[3 * (b - 1)];
        e[3 * b + 1] = e[3 * (b - 1) + 1];
        e[3 * b + 2] = e[3 * (b - 1) + 2];
        --b;
      }
      e[3 * b] = k0;
      e[3 * b + 1] = k1;
      e[3 * b + 2] = k2;
    }
    double sx = 0.0, sy = 0.0;
    for (unsigned a = 0; a < m; ++a) {
      sx += e[3 * a + 1];
      sy += e[3 * a + 2];
    }
    ctl->reaction_x = -sx;
    ctl->reaction_y = -sy;
    ctl->tool_work += (double)P.dt * (sx * P.ind_vx + sy * P.ind_vy);
    if (ctl->evals < (long long)P.load_cap) {
      B.load[2 * ctl->evals] = -sx;
      B.load[2 * ctl->evals + 1] = -sy;
    }
    ctl->load_entries = 0u;
  }
  const float vmax = sqrtf(__uint_as_float(atomicExch(&ctl->vmax2_bits, 0u)));
  ctl->ticket = 0;
  ctl->sp = sp ^ 1;
  ctl->evals += 1;
  const float disp = ctl->disp + vmax * (float)P.dt;
  ctl->disp = disp;
  const int rebuild = (disp > P.rebuild_disp) ? 1 : 0;
  ctl->rebuild_pending = rebuild;
  const int keep_going = (ctl->evals < ctl->target) && !(ctl->status & kStatusNonfinite);
  // use_cond bit 0: this launch sits in a graph with a rebuild IF node;
  // bit 1: it also sits in the step loop's WHILE body
  if (use_cond & 1) cudaGraphSetConditional(h_rebuild, (unsigned)rebuild);
  if (use_cond & 2) cudaGraphSetConditional(h_loop, (unsigned)keep_going);
}

// One thread per particle (variant 0) and the read-back kernel.
template <class T, int MODE, bool FEAT>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 4 : 2) force_kernel(Params<T> P, Bufs<T> B,
                                                            cudaGraphConditionalHandle h_rebuild,
                                                            cudaGraphConditionalHandle h_loop, int use_cond,
                                                            int primed) {
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  ThreadLedger<T> L;
  if (i < P.n) {
    const V4<T> p = B.pos[sp][i];
    const V4<T> v = B.vel[sp][i];
    const uint4 hd = B.head[lp][i];
    process_particle<T, MODE, FEAT>(P, B, sp, lp, i, p, v, hd, primed, B.ctl->evals, L);
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
  commit_epilogue<T, FEAT>(P, B, sp, L, h_rebuild, h_loop, use_cond);
}

// Persistent grid-stride variant: while a thread works on particle i it has
// the loads of its next particle already in flight (twice the memory-level
// parallelism of variant 0 at the cost of a dozen registers).
template <class T, int MODE, int BLOCK, int MINB, bool FEAT>
__global__ void __launch_bounds__(BLOCK, MINB) force_kernel_pf(Params<T> P, Bufs<T> B,
                                                               cudaGraphConditionalHandle h_rebuild,
                                                               cudaGraphConditionalHandle h_loop, int use_cond,
                                                               int primed) {
  static_assert(MODE != kPeek, "read-back uses force_kernel");
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const long long eval = B.ctl->evals;
  const int stride = gridDim.x * BLOCK;
  int i = blockIdx.x * BLOCK + threadIdx.x;
  ThreadLedger<T> L;
  V4<T> p{}, v{};
  uint4 hd = make_uint4(0u, 0u, 0u, 0u);
  if (i < P.n) {
    p = B.pos[sp][i];
    v = B.vel[sp][i];
    hd = B.head[lp][i];
  }
  while (i < P.n) {
    const int nx = i + stride;
    V4<T> pn{}, vn{};
    uint4 hn = make_uint4(0u, 0u, 0u, 0u);
    if (nx < P.n) {
      pn = B.pos[sp][nx];
      vn = B.vel[sp][nx];
      hn = B.head[lp][nx];
    }
    process_particle<T, MODE, FEAT>(P, B, sp, lp, i, p, v, hd, primed, eval, L);
    i = nx;
    p = pn;
    v = vn;
    hd = hn;
  }
  commit_epilogue<T, FEAT>(P, B, sp, L, h_rebuild, h_loop, use_cond);
}

// Bulk-copy variant: each block streams its tiles of own-particle state
// (position, velocity, list head: 48 B per particle in FP32) from HBM into
// shared memory with cp.async.bulk, double-buffered on two mbarriers, so the
// next tile is in flight while the current one is computed. Partner state is
// gathered from global memory (mostly L2 hits thanks to the cell sort).
constexpr long long kWaitBudget = 2000000000LL;  // ~1 s of SM clock per wait

template <class T, int MODE, int BLOCK, int MINB, bool FEAT>
__global__ void __launch_bounds__(BLOCK, MINB) force_kernel_bulk(Params<T> P, Bufs<T> B,
                                                                 cudaGraphConditionalHandle h_rebuild,
                                                                 cudaGraphConditionalHandle h_loop, int use_cond,
                                                                 int primed) {
  static_assert(MODE != kPeek, "read-back uses force_kernel");
  __shared__ alignas(128) V4<T> s_pos[2][BLOCK];
  __shared__ alignas(128) V4<T> s_vel[2][BLOCK];
  __shared__ alignas(128) uint4 s_head[2][BLOCK];
  __shared__ alignas(8) uint64_t s_bar[2];
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const long long eval = B.ctl->evals;
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
    const bool ok = bulk::mbar_wait_bounded(&s_bar[buf], (uint32_t)((k >> 1) & 1), kWaitBudget);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(&B.ctl->status, (int)kStatusTimeout);
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
  commit_epilogue<T, FEAT>(P, B, sp, L, h_rebuild, h_loop, use_cond);
}

// ---------------------------------------------------------------------------
// Rebuild pipeline. Every kernel is a no-op unless ctl->rebuild_pending.
// ---------------------------------------------------------------------------

// 1. new integer cell and offset of every particle; count per key.
template <class T>
__global__ void bin_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const int sp = ctl->sp;
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
  const T fx = floor(ox * P.inv_cell), fy = floor(oy * P.inv_cell);
  // clamp the shift so that a runaway particle cannot overflow the int maths
  const int kx = (int)fmin(fmax(fx, T(-65536)), T(65536));
  const int ky = (int)fmin(fmax(fy, T(-65536)), T(65536));
  const int nx = cx + kx, ny = cy + ky;
  const int cxn = min(max(nx, 0), P.ncx - 1), cyn = min(max(ny, 0), P.ncy - 1);
  if (nx < -1 || nx > P.ncx || ny < -1 || ny > P.ncy) status |= kStatusEscaped;
  const int sx = cxn - cx, sy = cyn - cy;
  const T nox = fma((T)(-sx), P.cell, ox);
  const T noy = fma((T)(-sy), P.cell, oy);
  B.tmp_cell[i] = cxn | (cyn << 16);
  B.tmp_off[i] = V2<T>{nox, noy};
  if (status) atomicOr(&ctl->status, status);
  atomicAdd(&B.cell_count[tile_key(cxn, cyn, P.tiles_x)], 1);
}

// 2. exclusive scan of the per-key counts (three phases, 4096 keys per block)
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

__global__ void scan_blocks_kernel(const Ctl* ctl, const int* in, int* out, int* block_sums, int n) {
  if (!ctl->rebuild_pending) return;
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

__global__ void scan_top_kernel(const Ctl* ctl, int* block_sums, int nblocks) {
  if (!ctl->rebuild_pending) return;
  // one block; nblocks <= kScanChunk
  const int base = threadIdx.x * kScanItems;
  int v[kScanItems];
  int local = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < nblocks) ? block_sums[base + k] : 0;
    local += v[k];
  }
  int total;
  int run = block_exclusive_scan(local, &total);
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < nblocks) block_sums[base + k] = run;
    run += v[k];
  }
}

__global__ void scan_add_kernel(const Ctl* ctl, int* out, const int* block_sums, int n) {
  if (!ctl->rebuild_pending) return;
  const int add = block_sums[blockIdx.x];
  const int base = blockIdx.x * kScanChunk;
  for (int k = threadIdx.x; k < kScanChunk; k += blockDim.x)
    if (base + k < n) out[base + k] += add;
}

// 3. scatter old indices into their key's range (order fixed by step 4)
template <class T>
__global__ void scatter_kernel(Params<T> P, Bufs<T> B) {
  if (!B.ctl->rebuild_pending) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const int c = B.tmp_cell[i];
  const int key = tile_key(c & 0xFFFF, c >> 16, P.tiles_x);
  const int slot = B.cell_start[key] + atomicAdd(&B.cell_fill[key], 1);
  B.perm[slot] = i;
}

// 4. deterministic order inside each cell: ascending original id
template <class T>
__global__ void cellsort_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  if (key >= P.nkeys) return;
  const int cnt = B.cell_count[key];
  if (cnt < 2) return;
  const int start = B.cell_start[key];
  const int* orig = B.orig[ctl->lp];
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

// 5. gather particle state into the new order (other buffers)
template <class T>
__global__ void gather_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int sp = ctl->sp, lp = ctl->lp;
  const int i = B.perm[p];
  const V4<T> q = B.pos[sp][i];
  const V2<T> off = B.tmp_off[i];
  B.pos[sp ^ 1][p] = V4<T>{off.x, off.y, q.z, cell_to_lane(B.tmp_cell[i], T(0))};
  B.vel[sp ^ 1][p] = B.vel[sp][i];
  B.orig[lp ^ 1][p] = B.orig[lp][i];
  B.invperm[i] = p;
  const size_t n = (size_t)P.n;
  for (int w = 0; w < 4; ++w) B.whist[lp ^ 1][w * n + p] = B.whist[lp][w * n + i];
}

// 5b. bond slots follow their disc; partners are renamed to the new order
template <class T>
__global__ void bond_gather_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending || P.BMAX == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int lp = ctl->lp;
  const int i = B.perm[p];
  const size_t n = (size_t)P.n;
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

// 6. candidate partners: the 3x3 cells around each particle, fixed order
template <class T>
__global__ void build_nbr_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int sp1 = ctl->sp ^ 1, lp1 = ctl->lp ^ 1;
  const V4<T>* pos = B.pos[sp1];
  unsigned* tail = B.nbr[lp1];
  unsigned first[kHeadSlots] = {0u, 0u, 0u};
  const V4<T> a = pos[p];
  const int c = lane_to_cell(a.w);
  const int cx = c & 0xFFFF, cy = c >> 16;
  const size_t n = (size_t)P.n;
  // bonded partners are handled through their bond slot (intact or broken)
  const int bc = P.BMAX > 0 ? B.bcnt[lp1][p] : 0;
  int cnt = 0;
  for (int dy = -1; dy <= 1; ++dy) {
    const int y = cy + dy;
    if (y < 0 || y >= P.ncy) continue;
    for (int dx = -1; dx <= 1; ++dx) {
      const int x = cx + dx;
      if (x < 0 || x >= P.ncx) continue;
      const int key = tile_key(x, y, P.tiles_x);
      const int start = B.cell_start[key];
      const int num = B.cell_count[key];
      for (int q = start; q < start + num; ++q) {
        if (q == p) continue;
        bool bonded = false;
        for (int t = 0; t < bc; ++t)
          if ((int)(B.bpart[lp1][(size_t)t * n + p] & kBondIdx) == q) bonded = true;
        if (bonded) continue;
        const V4<T> b = pos[q];
        const T ddx = fma((T)dx, P.cell, b.x - a.x);
        const T ddy = fma((T)dy, P.cell, b.y - a.y);
        const T reach = (a.z + b.z) + P.skin;
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
    atomicOr(&ctl->status, (int)kStatusCapacity);
    cnt = P.W;
  }
  B.head[lp1][p] = make_uint4((unsigned)cnt, first[0], first[1], first[2]);
  atomicMax(&ctl->max_cnt, cnt);
}

// 7. tangential-history remap keyed by the original-id pair: each particle
// looks its new partner up in its own old list (old sorted indices through
// perm) and carries the stored displacement over, flipping its sign when the
// pair's lower sorted index changed sides.
template <class T>
__global__ void link_kernel(Params<T> P, Bufs<T> B) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int lp = ctl->lp;
  const size_t n = (size_t)P.n;
  const unsigned* nbr = B.nbr[lp ^ 1];
  const unsigned* onbr = B.nbr[lp];
  const V2<T>* ohist = B.hist[lp];
  V2<T>* nhist = B.hist[lp ^ 1];
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

// 8. clear the key counters for the next rebuild
template <class T>
__global__ void clear_keys_kernel(Params<T> P, Bufs<T> B) {
  if (!B.ctl->rebuild_pending) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.nkeys) return;
  B.cell_count[k] = 0;
  B.cell_fill[k] = 0;
}

// 9. swap to the new buffers
__global__ void rebuild_flip_kernel(Ctl* ctl) {
  if (!ctl->rebuild_pending) return;
  ctl->sp ^= 1;
  ctl->lp ^= 1;
  ctl->disp = 0.0f;
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
  B.pos[sp][i] = V4<T>{(T)(x - cx * c), (T)(y - cy * c), (T)r, cell_to_lane(cx | (cy << 16), T(0))};
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
    pos[2 * o] = (double)(c & 0xFFFF) * cl + (double)q.x;
    pos[2 * o + 1] = (double)(c >> 16) * cl + (double)q.y;
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

__global__ void set_target_kernel(Ctl* ctl, long long n) { ctl->target = ctl->evals + n; }

__global__ void request_rebuild_kernel(Ctl* ctl) { ctl->rebuild_pending = 1; }

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

}  // namespace hm
}  // namespace tdem

// ===========================================================================
// Host engine
// ===========================================================================
namespace {

using namespace tdem::hm;

struct EngineBase {
  virtual ~EngineBase() = default;
  virtual int set_state(const double* pos, const double* vel, const double* omega, const double* radius,
                        const double* mass, const double* inertia, int host, cudaStream_t s) = 0;
  virtual int step(long long n, cudaStream_t s) = 0;
  virtual int read_state(double* pos, double* vel, double* omega, double* force, double* torque, int host,
                         cudaStream_t s) = 0;
  virtual int read_ledger(double* out, int count, cudaStream_t s) = 0;
  virtual int status(cudaStream_t s) = 0;
  virtual int read_pairs(int* out, long long capacity, long long* count, cudaStream_t s) = 0;
  virtual int use_graph(int on) = 0;
  virtual int set_variant(int v) = 0;
  virtual int set_bonds(const int* pairs, const double* strength, long long count, cudaStream_t s) = 0;
  virtual int read_bonds(int* pairs, int* state, long long capacity, long long* count, cudaStream_t s) = 0;
  virtual int read_load(double* out, long long capacity, long long* count, cudaStream_t s) = 0;
  virtual int step_kernel(cudaStream_t s) = 0;
  virtual int rebuild_pending(cudaStream_t s) = 0;
  virtual int get_variant() const = 0;
  virtual int autotune(int steps, cudaStream_t s, float* ms_out) = 0;
  virtual int rebuild(cudaStream_t s) = 0;
  virtual int read_history(int* pairs, double* xi, long long capacity, long long* count, cudaStream_t s) = 0;
  std::string err;
};

// Engine parameters from the public configuration (material constants as in
// oracle-independent closed forms: E* = E/(2(1-nu^2)), G* = E/(4(2-nu)(1+nu)),
// Tsuji beta from the restitution coefficient).
template <class T>
void make_params(const tdem_hm_config& c, int slots, Params<T>& P) {
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
  P.eps_t = c.breaking_strain;
  P.eps_s = c.shear_breaking_strain;
  P.ind_x0 = c.indenter_center[0];
  P.ind_y0 = c.indenter_center[1];
  P.ind_vx = c.indenter_velocity[0];
  P.ind_vy = c.indenter_velocity[1];
  P.irad = (T)c.indenter_radius;
  P.load_cap = c.indenter_radius > 0.0 ? std::max(c.load_capacity, 0) : 0;
}

// Bond slots from per-disc lists in original order (partner original id per
// slot, -1 for none): partners renamed to sorted indices, reference vectors
// from the current positions, and each disc's constant covariance pseudo-inverse.
template <class T>
__global__ void sorted_of_orig_kernel(Params<T> P, Bufs<T> B, int* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P.n) out[B.orig[B.ctl->lp][p]] = p;
}

template <class T>
__global__ void bond_init_kernel(Params<T> P, Bufs<T> B, const int* part_orig, const float* strength,
                                 const int* sorted_of_orig) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int sp = B.ctl->sp, lp = B.ctl->lp;
  const size_t n = (size_t)P.n;
  const int o = B.orig[lp][p];
  const V4<T> a = B.pos[sp][p];
  int bc = 0;
  T c00 = 0, c01 = 0, c11 = 0;
  for (int s = 0; s < P.BMAX; ++s) {
    const int qo = part_orig[(size_t)s * n + o];
    if (qo < 0) break;
    const int q = sorted_of_orig[qo];
    const V2<T> r = cell_delta<T>(P, a, B.pos[sp][q]);
    const size_t k = (size_t)s * n + p;
    B.bpart[lp][k] = (unsigned)q;
    B.bref[lp][k] = r;
    B.bstr[lp][k] = (T)strength[(size_t)s * n + o];
    B.bus[lp][k] = V2<T>{T(0), T(0)};
    B.bfail[lp][k] = -1;
    c00 += r.x * r.x;
    c01 += r.x * r.y;
    c11 += r.y * r.y;
    ++bc;
  }
  B.bcnt[lp][p] = bc;
  B.bpinv[lp][p] = pinv_sym2_dev<T>(c00, c01, c11);
}

// Bond states as original ids (lo, hi), read from the pair's lower sorted index.
template <class T>
__global__ void bonds_out_kernel(Params<T> P, Bufs<T> B, int* pairs, int* state, long long capacity,
                                 unsigned long long* count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int lp = B.ctl->lp;
  const size_t n = (size_t)P.n;
  const int bc = B.bcnt[lp][p];
  for (int s = 0; s < bc; ++s) {
    const size_t k = (size_t)s * n + p;
    const unsigned w = B.bpart[lp][k];
    const int q = (int)(w & kBondIdx);
    if (p >= q) continue;
    const unsigned long long e = atomicAdd(count, 1ull);
    if ((long long)e >= capacity) continue;
    const int a = B.orig[lp][p], b = B.orig[lp][q];
    pairs[2 * e] = min(a, b);
    pairs[2 * e + 1] = max(a, b);
    state[2 * e] = (w & kBondBroken) ? (int)((w >> kBondModeShift) & 3u) : 0;  // 0 intact, else mode
    state[2 * e + 1] = B.bfail[lp][k];
  }
}

// The rebuild pipeline (every kernel a no-op unless ctl->rebuild_pending).
template <class T>
void launch_rebuild_seq(const Params<T>& P, const Bufs<T>& B, cudaStream_t s) {
  const int nb = (P.n + kThreads - 1) / kThreads;
  const int nk = (P.nkeys + kThreads - 1) / kThreads;
  const int sb = (P.nkeys + kScanChunk - 1) / kScanChunk;
  bin_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  scan_blocks_kernel<<<sb, kScanThreads, 0, s>>>(B.ctl, B.cell_count, B.cell_start, B.block_sums, P.nkeys);
  scan_top_kernel<<<1, kScanThreads, 0, s>>>(B.ctl, B.block_sums, sb);
  scan_add_kernel<<<sb, kScanThreads, 0, s>>>(B.ctl, B.cell_start, B.block_sums, P.nkeys);
  scatter_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  cellsort_kernel<T><<<nk, kThreads, 0, s>>>(P, B);
  gather_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  bond_gather_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  build_nbr_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  link_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  clear_keys_kernel<T><<<nk, kThreads, 0, s>>>(P, B);
  rebuild_flip_kernel<<<1, 1, 0, s>>>(B.ctl);
}

// Step-kernel variants the autotuner chooses from: 0 = one thread per
// particle; 1..3 = persistent grid-stride with next-particle prefetch at three
// block shapes.
constexpr int kVariants = 6;

template <class T>
struct StepKernel {
  void* func;
  int block;
  int grid;
};

template <class T>
using StepFn = void (*)(Params<T>, Bufs<T>, cudaGraphConditionalHandle, cudaGraphConditionalHandle, int, int);

template <class T, bool F>
StepFn<T> step_fn_feat(int variant, int mode) {
  if (mode == kPrime) {
    switch (variant) {
      case 1: return &force_kernel_pf<T, kPrime, 256, 3, F>;
      case 2: return &force_kernel_pf<T, kPrime, 128, 6, F>;
      case 3: return &force_kernel_pf<T, kPrime, 256, 2, F>;
      case 4: return &force_kernel_bulk<T, kPrime, 256, 3, F>;
      case 5: return &force_kernel_bulk<T, kPrime, 128, 6, F>;
      default: return &force_kernel<T, kPrime, F>;
    }
  }
  switch (variant) {
    case 1: return &force_kernel_pf<T, kStep, 256, 3, F>;
    case 2: return &force_kernel_pf<T, kStep, 128, 6, F>;
    case 3: return &force_kernel_pf<T, kStep, 256, 2, F>;
    case 4: return &force_kernel_bulk<T, kStep, 256, 3, F>;
    case 5: return &force_kernel_bulk<T, kStep, 128, 6, F>;
    default: return &force_kernel<T, kStep, F>;
  }
}

// FEAT kernels carry the bonded-particle model and the indenter; the plain
// granular kernels compile without them (fewer registers).
template <class T>
StepFn<T> step_fn(int variant, int mode, bool feat) {
  return feat ? step_fn_feat<T, true>(variant, mode) : step_fn_feat<T, false>(variant, mode);
}

inline int variant_block(int variant) { return (variant == 2 || variant == 5) ? 128 : 256; }

template <class T>
struct Engine final : EngineBase {
  Params<T> P{};
  Bufs<T> B{};
  std::vector<void*> allocs;
  int nblocks = 0;
  int scan_blocks = 0;
  int variant = 0;
  int vgrid[kVariants] = {};
  int nwarp_slots = 0;
  bool primed = false;
  bool has_state = false;
  bool graph_on = true;
  bool graph_failed = false;
  std::string graph_error;
  cudaGraph_t graph = nullptr;       // n steps: WHILE loop
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph1 = nullptr;      // one step
  cudaGraphExec_t exec1 = nullptr;
  cudaGraphNode_t target_node = nullptr;
  long long exec_target = 0;
  cudaGraphConditionalHandle h_reb1 = 0;
  cudaStream_t cap_stream = nullptr;
  cudaGraphConditionalHandle h_loop = 0, h_reb = 0;
  double* stage = nullptr;        // device staging for host FP64 arrays
  double* host_stage = nullptr;   // pinned
  size_t stage_elems = 0;
  Ctl* host_ctl = nullptr;        // pinned mirror
  double* host_part = nullptr;    // pinned peek partials
  double* host_diss = nullptr;    // pinned committed partials
  double* host_frac = nullptr;    // pinned committed fracture partials

  ~Engine() override {
    destroy_graphs();
    if (cap_stream) cudaStreamDestroy(cap_stream);
    for (void* p : allocs) cudaFree(p);
    cudaFreeHost(host_stage);
    cudaFreeHost(host_ctl);
    cudaFreeHost(host_part);
    cudaFreeHost(host_diss);
    cudaFreeHost(host_frac);
  }

  void destroy_graphs() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (exec1) cudaGraphExecDestroy(exec1);
    if (graph1) cudaGraphDestroy(graph1);
    exec = exec1 = nullptr;
    graph = graph1 = nullptr;
  }

  template <class U>
  int alloc(U** p, size_t count) {
    void* q = nullptr;
    TDEM_CUDA_TRY(&err, cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(U)));
    TDEM_CUDA_TRY(&err, cudaMemset(q, 0, std::max<size_t>(1, count) * sizeof(U)));
    allocs.push_back(q);
    *p = static_cast<U*>(q);
    return TDEM_OK;
  }

  int init(const tdem_hm_config& c) {
    make_params<T>(c, c.max_neighbors, P);
    const size_t n = (size_t)c.n, W = (size_t)c.max_neighbors;
    nblocks = (int)((n + kThreads - 1) / kThreads);
    scan_blocks = (P.nkeys + kScanChunk - 1) / kScanChunk;
    // persistent variants: resident blocks per SM x SMs, never more than needed
    int dev = 0, sms = 1;
    TDEM_CUDA_TRY(&err, cudaGetDevice(&dev));
    TDEM_CUDA_TRY(&err, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    vgrid[0] = nblocks;
    nwarp_slots = nblocks * (kThreads / 32);
    for (int v = 1; v < kVariants; ++v) {
      int per_sm = 0;
      const int bs = variant_block(v);
      TDEM_CUDA_TRY(&err, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &per_sm, reinterpret_cast<const void*>(step_fn<T>(v, kStep, feat())), bs, 0));
      const int need = (int)((n + bs - 1) / bs);
      vgrid[v] = std::max(1, std::min(need, per_sm * sms));
      nwarp_slots = std::max(nwarp_slots, vgrid[v] * (bs / 32));
    }
    int rc = TDEM_OK;
    for (int b = 0; b < 2 && !rc; ++b) {
      if ((rc = alloc(&B.pos[b], n)) || (rc = alloc(&B.vel[b], n)) || (rc = alloc(&B.head[b], n)) ||
          (rc = alloc(&B.orig[b], n)) || (rc = alloc(&B.whist[b], 4 * n)) ||
          (rc = alloc(&B.nbr[b], (W > 3 ? W - 3 : 1) * n)) ||
          (rc = alloc(&B.hist[b], W * n)))
        return rc;
    }
    if ((rc = alloc(&B.cell_count, (size_t)P.nkeys)) || (rc = alloc(&B.cell_start, (size_t)P.nkeys)) ||
        (rc = alloc(&B.cell_fill, (size_t)P.nkeys)) || (rc = alloc(&B.perm, n)) ||
        (rc = alloc(&B.block_sums, (size_t)scan_blocks)) || (rc = alloc(&B.tmp_cell, n)) ||
        (rc = alloc(&B.tmp_off, n)) || (rc = alloc(&B.diss_part, (size_t)nwarp_slots)) ||
        (rc = alloc(&B.peek_part, (size_t)nblocks * 12)) || (rc = alloc(&B.peek_vel, n)) ||
        (rc = alloc(&B.peek_force, n)) || (rc = alloc(&B.ctl, 1)) || (rc = alloc(&B.invperm, n)) ||
        (rc = alloc(&B.frac_part, (size_t)nwarp_slots)) || (rc = alloc(&B.ind_part, 3 * (size_t)nwarp_slots)) ||
        (rc = alloc(&B.load, 2 * (size_t)std::max(P.load_cap, 1))))
      return rc;
    if (P.BMAX > 0) {
      const size_t BS = (size_t)P.BMAX * n;
      for (int b = 0; b < 2; ++b)
        if ((rc = alloc(&B.bpart[b], BS)) || (rc = alloc(&B.bref[b], BS)) || (rc = alloc(&B.bstr[b], BS)) ||
            (rc = alloc(&B.bus[b], BS)) || (rc = alloc(&B.bfail[b], BS)) || (rc = alloc(&B.bcnt[b], n)) ||
            (rc = alloc(&B.bpinv[b], n)))
          return rc;
      if ((rc = alloc(&B.strain, n))) return rc;
    }
    stage_elems = 8 * n;
    if ((rc = alloc(&stage, stage_elems))) return rc;
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_stage, stage_elems * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_ctl, sizeof(Ctl)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_part, (size_t)nblocks * 12 * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_frac, (size_t)nwarp_slots * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_diss, (size_t)nwarp_slots * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    return TDEM_OK;
  }

  bool feat() const { return P.BMAX > 0 || P.irad > T(0); }
  dim3 grid_n() const { return dim3((unsigned)nblocks); }
  dim3 grid_keys() const { return dim3((unsigned)((P.nkeys + kThreads - 1) / kThreads)); }

  void launch_rebuild(cudaStream_t s) { launch_rebuild_seq<T>(P, B, s); }

  int set_state(const double* pos, const double* vel, const double* omega, const double* radius,
                const double* mass, const double* inertia, int host, cudaStream_t s) override {
    const size_t n = (size_t)P.n;
    const double* d[6];
    if (host) {
      // stage through pinned memory: pos 2n, vel 2n, omega n, radius n, mass n, inertia n
      const double* src[6] = {pos, vel, omega, radius, mass, inertia};
      const size_t len[6] = {2 * n, 2 * n, n, n, n, n};
      size_t off = 0;
      for (int k = 0; k < 6; ++k) {
        if (!src[k]) return tdem::fail(&err, TDEM_ERR_BADARG, "set_state: null host array");
        std::memcpy(host_stage + off, src[k], len[k] * sizeof(double));
        d[k] = stage + off;
        off += len[k];
      }
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(stage, host_stage, off * sizeof(double), cudaMemcpyHostToDevice, s));
    } else {
      const double* src[6] = {pos, vel, omega, radius, mass, inertia};
      for (int k = 0; k < 6; ++k) {
        if (!src[k]) return tdem::fail(&err, TDEM_ERR_BADARG, "set_state: null device array");
        d[k] = src[k];
      }
    }
    Ctl zero{};
    zero.rebuild_pending = 1;
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(B.ctl, &zero, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    TDEM_CUDA_TRY(&err, cudaMemsetAsync(B.diss_part, 0, (size_t)nwarp_slots * sizeof(double), s));
    TDEM_CUDA_TRY(&err, cudaMemsetAsync(B.frac_part, 0, (size_t)nwarp_slots * sizeof(double), s));
    pack_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, d[0], d[1], d[2], d[3], d[4], d[5]);
    launch_rebuild(s);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    // the host copy must not be reused before the upload finished
    if (host) TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    primed = false;
    has_state = true;
    return TDEM_OK;
  }

  // Adds `kernel -> IF(h) { rebuild pipeline }` to graph g.
  int add_step_and_rebuild(cudaGraph_t g, const cudaGraphNode_t* dep, size_t ndep,
                           cudaGraphConditionalHandle h, cudaGraphConditionalHandle hl, int cond_bits) {
    int prim = 1;
    void* args[] = {&P, &B, &h, &hl, &cond_bits, &prim};
    cudaKernelNodeParams kp = {};
    kp.func = reinterpret_cast<void*>(step_fn<T>(variant, kStep, feat()));
    kp.gridDim = dim3((unsigned)vgrid[variant]);
    kp.blockDim = dim3((unsigned)variant_block(variant));
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    cudaGraphNode_t snode;
    if (P.BMAX > 0) {
      void* sargs[] = {&P, &B};
      cudaKernelNodeParams sk = {};
      sk.func = reinterpret_cast<void*>(&strain_kernel<T>);
      sk.gridDim = grid_n();
      sk.blockDim = dim3(kThreads);
      sk.kernelParams = sargs;
      TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&snode, g, dep, ndep, &sk));
      dep = &snode;
      ndep = 1;
    }
    cudaGraphNode_t knode;
    TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&knode, g, dep, ndep, &kp));
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = h;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode;
    TDEM_CUDA_TRY(&err, cudaGraphAddNode(&inode, g, &knode, nullptr, 1, &ip));
    cudaGraph_t rb = ip.conditional.phGraph_out[0];
    TDEM_CUDA_TRY(&err, cudaStreamBeginCaptureToGraph(cap_stream, rb, nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal));
    launch_rebuild(cap_stream);
    cudaGraph_t got = nullptr;
    TDEM_CUDA_TRY(&err, cudaStreamEndCapture(cap_stream, &got));
    return TDEM_OK;
  }

  // Two graphs: one step (kernel -> IF rebuild), and n steps
  // (set target -> WHILE { kernel -> IF rebuild }).
  int build_graph() {
    int rc;
    TDEM_CUDA_TRY(&err, cudaGraphCreate(&graph1, 0));
    TDEM_CUDA_TRY(&err, cudaGraphConditionalHandleCreate(&h_reb1, graph1, 0, cudaGraphCondAssignDefault));
    if ((rc = add_step_and_rebuild(graph1, nullptr, 0, h_reb1, 0, 1))) return rc;
    TDEM_CUDA_TRY(&err, cudaGraphInstantiate(&exec1, graph1, 0));

    TDEM_CUDA_TRY(&err, cudaGraphCreate(&graph, 0));
    TDEM_CUDA_TRY(&err, cudaGraphConditionalHandleCreate(&h_loop, graph, 1, cudaGraphCondAssignDefault));
    long long n0 = 1;
    void* targs[] = {&B.ctl, &n0};
    cudaKernelNodeParams tp = {};
    tp.func = reinterpret_cast<void*>(&set_target_kernel);
    tp.gridDim = dim3(1);
    tp.blockDim = dim3(1);
    tp.kernelParams = targs;
    TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&target_node, graph, nullptr, 0, &tp));
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    TDEM_CUDA_TRY(&err, cudaGraphAddNode(&wnode, graph, &target_node, nullptr, 1, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    TDEM_CUDA_TRY(&err, cudaGraphConditionalHandleCreate(&h_reb, body, 0, cudaGraphCondAssignDefault));
    if ((rc = add_step_and_rebuild(body, nullptr, 0, h_reb, h_loop, 3))) return rc;
    TDEM_CUDA_TRY(&err, cudaGraphInstantiate(&exec, graph, 0));
    exec_target = 1;
    return TDEM_OK;
  }

  // Point the n-step graph's target node at n (only when n changes).
  int set_graph_target(long long n) {
    if (n == exec_target) return TDEM_OK;
    long long nn = n;
    void* targs[] = {&B.ctl, &nn};
    cudaKernelNodeParams tp = {};
    tp.func = reinterpret_cast<void*>(&set_target_kernel);
    tp.gridDim = dim3(1);
    tp.blockDim = dim3(1);
    tp.kernelParams = targs;
    TDEM_CUDA_TRY(&err, cudaGraphExecKernelNodeSetParams(exec, target_node, &tp));
    exec_target = n;
    return TDEM_OK;
  }

  void launch_strain(cudaStream_t s) {
    if (P.BMAX > 0) strain_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B);
  }

  int prime(cudaStream_t s) {
    launch_strain(s);
    step_fn<T>(variant, kPrime, feat())<<<vgrid[variant], variant_block(variant), 0, s>>>(P, B, 0, 0, 0, 1);
    launch_rebuild(s);  // runs only if the prime step tripped the trigger
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    primed = true;
    return TDEM_OK;
  }

  int step(long long n, cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "step before set_state");
    if (n <= 0) return TDEM_OK;
    if (!primed) {
      int rc = prime(s);
      if (rc) return rc;
      --n;
      if (n == 0) return TDEM_OK;
    }
    if (graph_on && !graph_failed && !exec) {
      if (build_graph() != TDEM_OK) {
        // fall back to plain launches (same kernels, same results)
        graph_error = err;
        graph_failed = true;
        destroy_graphs();
        cudaGetLastError();
      }
    }
    if (graph_on && exec) {
      if (n == 1) {
        TDEM_CUDA_TRY(&err, cudaGraphLaunch(exec1, s));
        return TDEM_OK;
      }
      int rc = set_graph_target(n);
      if (rc) return rc;
      TDEM_CUDA_TRY(&err, cudaGraphLaunch(exec, s));
      return TDEM_OK;
    }
    for (long long k = 0; k < n; ++k) {
      launch_strain(s);
      step_fn<T>(variant, kStep, feat())<<<vgrid[variant], variant_block(variant), 0, s>>>(P, B, 0, 0, 0, 1);
      launch_rebuild(s);
    }
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int peek(cudaStream_t s) {
    launch_strain(s);
    if (feat())
      force_kernel<T, kPeek, true><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, primed ? 1 : 0);
    else
      force_kernel<T, kPeek, false><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, primed ? 1 : 0);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read_state(double* pos, double* vel, double* omega, double* force, double* torque, int host,
                 cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "read before set_state");
    int rc = peek(s);
    if (rc) return rc;
    const size_t n = (size_t)P.n;
    if (host) {
      double* d = stage;  // pos 2n, vel 2n, omega n, force 2n, torque n
      unpack_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, d, d + 2 * n, d + 4 * n, d + 5 * n, d + 7 * n);
      TDEM_CUDA_TRY(&err, cudaGetLastError());
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_stage, stage, 8 * n * sizeof(double), cudaMemcpyDeviceToHost, s));
      TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
      if (pos) std::memcpy(pos, host_stage, 2 * n * sizeof(double));
      if (vel) std::memcpy(vel, host_stage + 2 * n, 2 * n * sizeof(double));
      if (omega) std::memcpy(omega, host_stage + 4 * n, n * sizeof(double));
      if (force) std::memcpy(force, host_stage + 5 * n, 2 * n * sizeof(double));
      if (torque) std::memcpy(torque, host_stage + 7 * n, n * sizeof(double));
      return TDEM_OK;
    }
    unpack_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, pos, vel, omega, force, torque);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read_ledger(double* out, int count, cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "read before set_state");
    int rc = peek(s);
    if (rc) return rc;
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_part, B.peek_part, (size_t)nblocks * 12 * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_frac, B.frac_part, (size_t)nwarp_slots * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
    const int nwarps = nwarp_slots;
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_diss, B.diss_part, (size_t)nwarps * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    // Neumaier-compensated sums in block order
    double v[TDEM_HM_L_COUNT] = {0};
    auto csum = [&](auto get, int count) {
      double sum = 0.0, comp = 0.0;
      for (int b = 0; b < count; ++b) {
        const double x = get(b);
        const double t = sum + x;
        comp += (std::fabs(sum) >= std::fabs(x)) ? (sum - t) + x : (x - t) + sum;
        sum = t;
      }
      return sum + comp;
    };
    double part[9];
    for (int k = 0; k < 9; ++k) part[k] = csum([&](int b) { return host_part[(size_t)b * 12 + k]; }, nblocks);
    for (int k = 0; k < 4; ++k) v[k] = part[k];
    v[TDEM_HM_L_DISSIPATED] = csum([&](int b) { return host_diss[b]; }, nwarps) + part[4];
    v[TDEM_HM_L_BOND_ELASTIC] = part[5];
    v[TDEM_HM_L_FRACTURE] = csum([&](int b) { return host_frac[b]; }, nwarps) + part[6];
    v[TDEM_HM_L_TOOL_WORK] = host_ctl->tool_work + (primed ? part[7] : 0.0);
    v[TDEM_HM_L_BROKEN] = (double)host_ctl->broken + part[8];
    v[TDEM_HM_L_TOTAL] = v[TDEM_HM_L_KINETIC] + v[TDEM_HM_L_POTENTIAL] + v[TDEM_HM_L_HERTZ] +
                         v[TDEM_HM_L_TANGENTIAL] + v[TDEM_HM_L_DISSIPATED] + v[TDEM_HM_L_BOND_ELASTIC] +
                         v[TDEM_HM_L_FRACTURE] - v[TDEM_HM_L_TOOL_WORK];
    v[TDEM_HM_L_EVALS] = (double)host_ctl->evals;
    v[TDEM_HM_L_REBUILDS] = (double)host_ctl->rebuilds;
    v[TDEM_HM_L_MAX_NEIGHBORS] = (double)host_ctl->max_cnt;
    v[TDEM_HM_L_STATUS] = (double)host_ctl->status;
    v[TDEM_HM_L_GRAPH] = (exec != nullptr) ? 1.0 : 0.0;
    v[TDEM_HM_L_VARIANT] = (double)variant;
    std::memcpy(out, v, std::min(count, (int)TDEM_HM_L_COUNT) * sizeof(double));
    return TDEM_OK;
  }

  int status(cudaStream_t s) override {
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    const int st = host_ctl->status;
    if (st & kStatusNonfinite) return tdem::fail(&err, TDEM_ERR_NONFINITE, "non-finite particle state; reduce dt");
    if (st & kStatusCapacity)
      return tdem::fail(&err, TDEM_ERR_CAPACITY,
                        "neighbour capacity exceeded (max_neighbors=" + std::to_string(P.W) + ")");
    if (st & kStatusEscaped) return tdem::fail(&err, TDEM_ERR_CAPACITY, "a particle left the cell grid");
    if (st & kStatusTimeout) return tdem::fail(&err, TDEM_ERR_CUDA, "a bounded wait on a bulk copy timed out");
    if (st & kStatusInertia)
      return tdem::fail(&err, TDEM_ERR_BADARG, "moment of inertia must be inertia_factor * m * r^2");
    return TDEM_OK;
  }

  int read_pairs(int* out, long long capacity, long long* count, cudaStream_t s) override {
    unsigned long long* dcount = nullptr;
    int* dout = nullptr;
    TDEM_CUDA_TRY(&err, cudaMalloc(&dcount, sizeof(unsigned long long)));
    TDEM_CUDA_TRY(&err, cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dout, std::max<long long>(1, capacity) * 2 * sizeof(int)));
    pairs_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, dout, capacity, dcount);
    unsigned long long c = 0;
    cudaMemcpyAsync(&c, dcount, sizeof(c), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const long long m = std::min<long long>((long long)c, capacity);
    if (m > 0) cudaMemcpy(out, dout, (size_t)m * 2 * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dcount);
    cudaFree(dout);
    *count = (long long)c;
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int use_graph(int on) override {
    graph_on = on != 0;
    return TDEM_OK;
  }

  int step_kernel(cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "step before set_state");
    if (!primed) return prime(s);
    launch_strain(s);
    step_fn<T>(variant, kStep, feat())<<<vgrid[variant], variant_block(variant), 0, s>>>(P, B, 0, 0, 0, 1);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int rebuild_pending(cudaStream_t s) override {
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    return host_ctl->rebuild_pending ? 1 : 0;
  }

  int set_bonds(const int* pairs, const double* strength, long long count, cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "set_bonds before set_state");
    if (P.BMAX <= 0) return tdem::fail(&err, TDEM_ERR_BADARG, "engine created with max_bonds = 0");
    if (primed) return tdem::fail(&err, TDEM_ERR_STATE, "set_bonds must follow set_state, before stepping");
    const size_t n = (size_t)P.n;
    std::vector<int> part((size_t)P.BMAX * n, -1);
    std::vector<float> str((size_t)P.BMAX * n, 1.0f);
    std::vector<int> fill(n, 0);
    for (long long b = 0; b < count; ++b) {
      const int a = pairs[2 * b], c = pairs[2 * b + 1];
      if (a < 0 || c < 0 || a >= P.n || c >= P.n || a == c)
        return tdem::fail(&err, TDEM_ERR_BADARG, "bond " + std::to_string(b) + " has an invalid disc index");
      if (!(strength[b] > 0.0)) return tdem::fail(&err, TDEM_ERR_BADARG, "bond strength factors must be positive");
      for (int e : {a, c}) {
        const int o = e == a ? c : a;
        if (fill[e] >= P.BMAX)
          return tdem::fail(&err, TDEM_ERR_BADARG,
                            "disc " + std::to_string(e) + " has more than max_bonds = " + std::to_string(P.BMAX) +
                                " bonds");
        part[(size_t)fill[e] * n + e] = o;
        str[(size_t)fill[e] * n + e] = (float)strength[b];
        ++fill[e];
      }
    }
    int* dpart = nullptr;
    float* dstr = nullptr;
    TDEM_CUDA_TRY(&err, cudaMalloc(&dpart, part.size() * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dstr, str.size() * sizeof(float)));
    cudaMemcpyAsync(dpart, part.data(), part.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dstr, str.data(), str.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    sorted_of_orig_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, B.invperm);
    bond_init_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, dpart, dstr, B.invperm);
    const cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(dpart);
    cudaFree(dstr);
    TDEM_CUDA_TRY(&err, e);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    // bonded pairs leave the contact candidates: rebuild the list now
    request_rebuild_kernel<<<1, 1, 0, s>>>(B.ctl);
    launch_rebuild(s);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read_bonds(int* pairs, int* state, long long capacity, long long* count, cudaStream_t s) override {
    if (P.BMAX <= 0) {
      *count = 0;
      return TDEM_OK;
    }
    unsigned long long* dcount = nullptr;
    int *dpairs = nullptr, *dstate = nullptr;
    const size_t cap = (size_t)std::max<long long>(1, capacity);
    TDEM_CUDA_TRY(&err, cudaMalloc(&dcount, sizeof(unsigned long long)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dpairs, cap * 2 * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dstate, cap * 2 * sizeof(int)));
    cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
    bonds_out_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, dpairs, dstate, capacity, dcount);
    unsigned long long c = 0;
    cudaMemcpyAsync(&c, dcount, sizeof(c), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const size_t m = (size_t)std::min<long long>((long long)c, capacity);
    if (m) {
      cudaMemcpy(pairs, dpairs, m * 2 * sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemcpy(state, dstate, m * 2 * sizeof(int), cudaMemcpyDeviceToHost);
    }
    cudaFree(dcount);
    cudaFree(dpairs);
    cudaFree(dstate);
    *count = (long long)c;
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read_load(double* out, long long capacity, long long* count, cudaStream_t s) override {
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    const long long have = std::min<long long>(host_ctl->evals, (long long)P.load_cap);
    const long long m = std::min(have, capacity);
    if (m > 0) TDEM_CUDA_TRY(&err, cudaMemcpy(out, B.load, (size_t)m * 2 * sizeof(double), cudaMemcpyDeviceToHost));
    *count = have;
    return TDEM_OK;
  }

  int set_variant(int v) override {
    if (v < 0 || v >= kVariants) return tdem::fail(&err, TDEM_ERR_BADARG, "unknown step-kernel variant");
    if (v != variant) {
      variant = v;
      destroy_graphs();
    }
    return TDEM_OK;
  }

  int get_variant() const override { return variant; }

  // Time `steps` steps with every variant (advancing the simulation) and keep
  // the fastest. Per-particle arithmetic is identical in all variants.
  int autotune(int steps, cudaStream_t s, float* ms_out) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "autotune before set_state");
    cudaEvent_t e0, e1;
    TDEM_CUDA_TRY(&err, cudaEventCreate(&e0));
    TDEM_CUDA_TRY(&err, cudaEventCreate(&e1));
    int best = variant;
    float best_ms = 1e30f;
    for (int v = 0; v < kVariants; ++v) {
      int rc = set_variant(v);
      if (!rc) rc = step(2, s);  // builds the graph outside the timing
      if (rc) return rc;
      TDEM_CUDA_TRY(&err, cudaEventRecord(e0, s));
      if ((rc = step(steps, s))) return rc;
      TDEM_CUDA_TRY(&err, cudaEventRecord(e1, s));
      TDEM_CUDA_TRY(&err, cudaEventSynchronize(e1));
      float ms = 0.0f;
      TDEM_CUDA_TRY(&err, cudaEventElapsedTime(&ms, e0, e1));
      if (ms_out) ms_out[v] = ms;
      if (ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return set_variant(best);
  }

  int rebuild(cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "rebuild before set_state");
    request_rebuild_kernel<<<1, 1, 0, s>>>(B.ctl);
    launch_rebuild(s);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read_history(int* pairs, double* xi, long long capacity, long long* count, cudaStream_t s) override {
    unsigned long long* dcount = nullptr;
    int* dpairs = nullptr;
    double* dxi = nullptr;
    const size_t cap = (size_t)std::max<long long>(1, capacity);
    TDEM_CUDA_TRY(&err, cudaMalloc(&dcount, sizeof(unsigned long long)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dpairs, cap * 2 * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&dxi, cap * 2 * sizeof(double)));
    cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
    history_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, dpairs, dxi, capacity, dcount);
    unsigned long long c = 0;
    cudaMemcpyAsync(&c, dcount, sizeof(c), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const size_t m = (size_t)std::min<long long>((long long)c, capacity);
    if (m) {
      cudaMemcpy(pairs, dpairs, m * 2 * sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemcpy(xi, dxi, m * 2 * sizeof(double), cudaMemcpyDeviceToHost);
    }
    cudaFree(dcount);
    cudaFree(dpairs);
    cudaFree(dxi);
    *count = (long long)c;
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }
};

std::string g_hm_create_error;

}  // namespace

struct tdem_hm {
  std::unique_ptr<EngineBase> e;
};

extern "C" {

int tdem_hm_create(const tdem_hm_config* c, tdem_hm** out) {
  g_hm_create_error.clear();
  std::string* err = &g_hm_create_error;
  if (!c || !out) return tdem::fail(err, TDEM_ERR_BADARG, "null argument");
  *out = nullptr;
  if (c->n < 1) return tdem::fail(err, TDEM_ERR_BADARG, "n out of range");
  if (c->max_neighbors < 1 || c->max_neighbors > kMaxSlots)
    return tdem::fail(err, TDEM_ERR_BADARG, "max_neighbors must be in 1..24");
  if (!(c->inertia_factor > 0.0)) return tdem::fail(err, TDEM_ERR_BADARG, "inertia_factor must be positive");
  if (c->max_bonds < 0 || c->max_bonds > kMaxBondSlots)
    return tdem::fail(err, TDEM_ERR_BADARG, "max_bonds must be in 0..8");
  if (c->max_bonds > 0 && (!(c->bond_kn > 0) || !(c->bond_ks >= 0) || !(c->bond_damping >= 0) ||
                           !(c->breaking_strain > 0) || !(c->shear_breaking_strain > 0)))
    return tdem::fail(err, TDEM_ERR_BADARG, "invalid bond stiffness, damping or break strain");
  if (!(c->indenter_radius >= 0)) return tdem::fail(err, TDEM_ERR_BADARG, "indenter_radius must be >= 0");
  if (c->ncx < 1 || c->ncy < 1 || c->ncx > 32768 || c->ncy > 32768)
    return tdem::fail(err, TDEM_ERR_BADARG, "cell grid must be 1..32768 per axis");
  if (!(c->cell > 0) || !(c->skin >= 0) || !(c->dt > 0) || !(c->young > 0) || !(c->poisson > -1.0) ||
      !(c->poisson < 0.5) || !(c->restitution > 0) || !(c->restitution <= 1) || !(c->mu >= 0) ||
      !(c->mu_wall >= 0))
    return tdem::fail(err, TDEM_ERR_BADARG, "invalid material, cell or time-step parameter");
  if (c->precision != 32 && c->precision != 64)
    return tdem::fail(err, TDEM_ERR_BADARG, "precision must be 32 or 64");
  auto* h = new tdem_hm();
  int rc;
  if (c->precision == 32) {
    auto* e = new Engine<float>();
    h->e.reset(e);
    rc = e->init(*c);
  } else {
    auto* e = new Engine<double>();
    h->e.reset(e);
    rc = e->init(*c);
  }
  if (rc) {
    *err = h->e->err;
    delete h;
    return rc;
  }
  *out = h;
  return TDEM_OK;
}

void tdem_hm_destroy(tdem_hm* h) { delete h; }

int tdem_hm_set_state(tdem_hm* h, const double* pos, const double* vel, const double* omega, const double* radius,
                      const double* mass, const double* inertia, int host, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->set_state(pos, vel, omega, radius, mass, inertia, host, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_step(tdem_hm* h, int64_t n_steps, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->step((long long)n_steps, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_read_state(tdem_hm* h, double* pos, double* vel, double* omega, double* force, double* torque,
                       int host, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->read_state(pos, vel, omega, force, torque, host, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_read_ledger(tdem_hm* h, double* out, int count, void* stream) {
  if (!h || !out || count < 0) return TDEM_ERR_BADARG;
  return h->e->read_ledger(out, count, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_status(tdem_hm* h, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->status(reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_read_pairs(tdem_hm* h, int32_t* out, int64_t capacity, int64_t* count, void* stream) {
  if (!h || !out || !count) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->read_pairs(out, (long long)capacity, &c, reinterpret_cast<cudaStream_t>(stream));
  *count = (int64_t)c;
  return rc;
}

int tdem_hm_rebuild(tdem_hm* h, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->rebuild(reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_read_history(tdem_hm* h, int32_t* pairs, double* xi, int64_t capacity, int64_t* count,
                         void* stream) {
  if (!h || !pairs || !xi || !count) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->read_history(pairs, xi, (long long)capacity, &c, reinterpret_cast<cudaStream_t>(stream));
  *count = (int64_t)c;
  return rc;
}

int tdem_hm_set_bonds(tdem_hm* h, const int32_t* pairs, const double* strength, int64_t count, void* stream) {
  if (!h || (count > 0 && (!pairs || !strength)) || count < 0) return TDEM_ERR_BADARG;
  return h->e->set_bonds(pairs, strength, (long long)count, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_read_bonds(tdem_hm* h, int32_t* pairs, int32_t* state, int64_t capacity, int64_t* count,
                       void* stream) {
  if (!h || !pairs || !state || !count) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->read_bonds(pairs, state, (long long)capacity, &c, reinterpret_cast<cudaStream_t>(stream));
  *count = (int64_t)c;
  return rc;
}

int tdem_hm_read_load(tdem_hm* h, double* out, int64_t capacity, int64_t* count, void* stream) {
  if (!h || !out || !count) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->read_load(out, (long long)capacity, &c, reinterpret_cast<cudaStream_t>(stream));
  *count = (int64_t)c;
  return rc;
}

int tdem_hm_step_kernel(tdem_hm* h, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->step_kernel(reinterpret_cast<cudaStream_t>(stream));
}

int tdem_hm_rebuild_pending(tdem_hm* h, void* stream) {
  if (!h) return -TDEM_ERR_BADARG;
  const int r = h->e->rebuild_pending(reinterpret_cast<cudaStream_t>(stream));
  return r;
}

int tdem_hm_num_variants(void) { return kVariants; }

int tdem_hm_set_variant(tdem_hm* h, int variant) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->set_variant(variant);
}

int tdem_hm_get_variant(const tdem_hm* h) { return h ? h->e->get_variant() : -1; }

int tdem_hm_autotune(tdem_hm* h, int steps, float* ms_out, void* stream) {
  if (!h || steps < 1) return TDEM_ERR_BADARG;
  return h->e->autotune(steps, reinterpret_cast<cudaStream_t>(stream), ms_out);
}

int tdem_hm_use_graph(tdem_hm* h, int on) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->use_graph(on);
}

int tdem_hm_last_error(const tdem_hm* h, char* buf, size_t len) {
  if (!buf || len == 0) return TDEM_ERR_BADARG;
  const std::string& e = h ? h->e->err : g_hm_create_error;
  const size_t m = std::min(len - 1, e.size());
  std::memcpy(buf, e.data(), m);
  buf[m] = '\0';
  return TDEM_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free contact-force evaluation
//
// For callers that must not allocate device memory: code that runs while
// another solver's CUDA graph is being captured (a cudaMalloc there breaks
// the capture), host callbacks and real-time coupling loops where an
// allocation's latency or failure is not acceptable, and plug-ins whose host
// application owns all device memory. The scratch lives in one file-scope
// device array that every GPU loading this library holds until the process
// exits.
// ===========================================================================
namespace {

constexpr int kNoAllocMaxDiscs = 16384;      // discs per call
constexpr int kNoAllocSlots = 8;             // candidate partners per disc
constexpr int kNoAllocMaxKeys = 65536;       // cell keys: grids up to 256 x 256 cells
constexpr size_t kNoAllocBytes = 8u << 20;   // 8 MiB

}  // namespace

static __device__ __align__(256) unsigned char tdem_noalloc_scratch[kNoAllocBytes];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_base[kNoAllocMaxDevices] = {};

// Bump carving of the scratch array, 256-byte aligned pieces.
struct Carver {
  unsigned char* base;
  size_t off;
  size_t cap;
  template <class U>
  U* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    U* p = reinterpret_cast<U*>(base + off);
    off += std::max<size_t>(1, count) * sizeof(U);
    return p;
  }
};

__global__ void noalloc_clear_kernel(Ctl* ctl, int* cell_count, int* cell_fill, int nkeys) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nkeys) {
    cell_count[k] = 0;
    cell_fill[k] = 0;
  }
  if (k == 0) {
    Ctl z{};
    z.rebuild_pending = 1;
    *ctl = z;
  }
}

__global__ void noalloc_status_kernel(const Ctl* ctl, int* status_out) { *status_out = ctl->status; }

// Error text into the caller's buffer, without touching the heap.
int noalloc_fail(char* buf, size_t len, int code, const char* fmt, long long a = 0, long long b = 0) {
  if (buf && len) snprintf(buf, len, fmt, a, b);
  return code;
}

}  // namespace

extern "C" {

int tdem_hm_contact_forces_noalloc(const tdem_hm_config* cfg, const double* pos, const double* vel,
                                   const double* omega, const double* radius, const double* mass,
                                   const double* inertia, double* out_force, double* out_torque, char* err_buf,
                                   size_t err_len, void* stream) {
  if (err_buf && err_len) err_buf[0] = '\0';
  if (!cfg || !pos || !vel || !omega || !radius || !mass || !inertia || !out_force || !out_torque)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG, "null argument");
  if (cfg->precision != 32)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG, "the allocation-free path is FP32 only");
  if (cfg->n < 1 || cfg->n > kNoAllocMaxDiscs)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG,
                        "the allocation-free path holds at most %lld discs per call, got %lld",
                        (long long)kNoAllocMaxDiscs, (long long)cfg->n);
  if (cfg->ncx < 1 || cfg->ncy < 1 || !(cfg->cell > 0) || !(cfg->inertia_factor > 0) || !(cfg->young > 0) ||
      !(cfg->restitution > 0) || !(cfg->restitution <= 1) || !(cfg->poisson > -1.0) || !(cfg->poisson < 0.5))
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG, "invalid cell grid or material");
  Params<float> P{};
  make_params<float>(*cfg, kNoAllocSlots, P);
  P.BMAX = 0;  // contacts, walls and gravity only: no bond slots live in the scratch
  P.irad = 0.0f;
  P.load_cap = 0;
  if (P.nkeys > kNoAllocMaxKeys)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG,
                        "the allocation-free path holds cell grids up to 256 x 256 cells; this grid is %lld x %lld",
                        (long long)cfg->ncx, (long long)cfg->ncy);
  // device address of the scratch array, resolved once per device
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_CUDA, "cannot query the current device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, tdem_noalloc_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(err_buf, err_len, TDEM_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed (%lld)",
                            (long long)e);
      g_noalloc_base[dev] = p;
    }
    base = g_noalloc_base[dev];
  }
  const size_t n = (size_t)cfg->n;
  const size_t W = kNoAllocSlots;
  const int nb = (int)((n + kThreads - 1) / kThreads);
  const int sb = (P.nkeys + kScanChunk - 1) / kScanChunk;
  Carver c{static_cast<unsigned char*>(base), 0, kNoAllocBytes};
  Bufs<float> B{};
  for (int b = 0; b < 2; ++b) {
    B.pos[b] = c.take<V4<float>>(n);
    B.vel[b] = c.take<V4<float>>(n);
    B.head[b] = c.take<uint4>(n);
    B.nbr[b] = c.take<unsigned>((W - kHeadSlots) * n);
    B.hist[b] = c.take<V2<float>>(W * n);
    B.orig[b] = c.take<int>(n);
    B.whist[b] = c.take<V2<float>>(4 * n);
  }
  B.cell_count = c.take<int>((size_t)P.nkeys);
  B.cell_start = c.take<int>((size_t)P.nkeys);
  B.cell_fill = c.take<int>((size_t)P.nkeys);
  B.perm = c.take<int>(n);
  B.block_sums = c.take<int>((size_t)sb);
  B.tmp_cell = c.take<int>(n);
  B.tmp_off = c.take<V2<float>>(n);
  B.diss_part = c.take<double>((size_t)nb * (kThreads / 32));
  B.peek_part = c.take<double>((size_t)nb * 12);
  B.peek_vel = c.take<V4<float>>(n);
  B.peek_force = c.take<V4<float>>(n);
  B.invperm = c.take<int>(n);
  B.ctl = c.take<Ctl>(1);
  int* status_dev = c.take<int>(1);
  if (c.off > c.cap)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_CAPACITY, "scratch too small: %lld of %lld bytes needed",
                        (long long)c.off, (long long)c.cap);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: clear what must start at zero
  noalloc_clear_kernel<<<(P.nkeys + kThreads - 1) / kThreads, kThreads, 0, s>>>(B.ctl, B.cell_count,
                                                                               B.cell_fill, P.nkeys);
  pack_kernel<float><<<nb, kThreads, 0, s>>>(P, B, pos, vel, omega, radius, mass, inertia);
  launch_rebuild_seq<float>(P, B, s);
  force_kernel<float, kPeek, false><<<nb, kThreads, 0, s>>>(P, B, 0, 0, 0, 0);
  unpack_kernel<float><<<nb, kThreads, 0, s>>>(P, B, nullptr, nullptr, nullptr, out_force, out_torque);
  noalloc_status_kernel<<<1, 1, 0, s>>>(B.ctl, status_dev);
  cudaError_t e = cudaGetLastError();
  int status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, status_dev, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_CUDA, "CUDA error %lld during the evaluation", (long long)e);
  if (status & kStatusNonfinite) return noalloc_fail(err_buf, err_len, TDEM_ERR_NONFINITE, "non-finite disc state");
  if (status & kStatusCapacity)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_CAPACITY, "a disc has more than %lld candidate partners",
                        (long long)kNoAllocSlots);
  if (status & kStatusEscaped)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_CAPACITY, "a disc lies outside the cell grid");
  if (status & kStatusInertia)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG, "moment of inertia must be inertia_factor * m * r^2");
  return TDEM_OK;
}

}  // extern "C"
