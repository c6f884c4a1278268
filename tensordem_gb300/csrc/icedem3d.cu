// 3-D reference mode: the FP64 bonded-sphere step of the reference's IceDEM3D
// (src/tensordem/dem3d.py:564-1663), on sm_103a.
//
// Design. One cooperative launch runs many steps of one instance on all SMs.
// This part's FP64 pipes are narrow (tens of cycles per warp-wide FP64
// instruction), so a step is as long as its longest per-thread FP64 chain:
// the work is cut so that no thread carries more than one particle's share of
// one sum, without reordering any sum. Five phases per step, separated by a
// grid barrier with a bounded wait; every scratch array lives in the handle.
// Cells are cell = floor(x / 2r) keyed into open-addressing tables
// (dem3d.py:825-856 builds the same cells in a dict); there are two tables,
// by step parity, so a step's positions are hashed at the end of the step
// before.
//   A. cell ranges of this step's table from an atomic cursor; the other
//      table cleared; objective shear strain (dem3d.py:875-901), a 16-lane
//      group per particle, lane w summing component w of the bond sum in the
//      bond list's order;
//   B. bond force, break test and commit, Maxwell branches, creep clock, one
//      thread per bond (dem3d.py:984-1100, 1342-1360); members into cells;
//   C1. each particle lists its overlapping partners with higher ids in the
//      reference's pair-list order: cells in offset order, members ascending
//      (lookups of nine cells in flight together);
//   C2. one thread per overlapping pair: normal force, friction with the
//      pair's history, rolling couple (dem3d.py:1382-1514); the partner gets
//      the pair in its inbox with the key of the reference's order for its
//      side (first particle of this particle's cell, then this particle);
//   D. assembly and semi-implicit Euler, four lanes per particle, lane w
//      summing force component w in the order of the reference's index_add_
//      calls (bond i-side then j-side, then per contact term its own pairs
//      then its sorted inbox), then tool, platens and integration
//      (dem3d.py:1516-1663); the new positions go into the other table.
// Pair forces that the reference adds as exact zeros are skipped. Every value
// a particle or bond gets is computed by one thread, independent of the grid,
// so trajectories are bitwise reproducible; ledger sums combine per-block
// partials in block order.
//
// This translation unit is compiled with --fmad=false: the reference runs
// one torch op per arithmetic step, each rounded separately.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"

namespace tdem {
namespace icedem3d {

constexpr int kMaxParticles = 1 << 20;
constexpr int kBlock = 128;               // threads per block
constexpr int kItemsPerBlock = 32;        // grid sizing: at most this many items per block
constexpr unsigned long long kBarrierSpins = 1ull << 24;  // ~1 s of 64 ns naps
constexpr int kContacts = 32;  // overlapping partners of one particle, per side
constexpr int kHistory = 64;   // friction-history entries of one particle (as the pair's lower id)
constexpr long long kCoordHalf = 1ll << 20;  // |cell coordinate| bound of the 21-bit packing
constexpr unsigned long long kEmpty = ~0ull;
constexpr double kEps = 2.220446049250313e-16;

constexpr int kStatusNonfinite = 1;
constexpr int kStatusContacts = 2;
constexpr int kStatusHistory = 4;
constexpr int kStatusEscaped = 8;
constexpr int kStatusBarrier = 16;
constexpr int kPartials = 16;  // per-block ledger partial sums

struct Dev {
  // topology (constant)
  const int* bi;
  const int* bj;
  const double* rest;
  const double* ref;    // (B,3)
  const double* inorm;  // (B,3)
  const double* thr;    // (B) or null
  const double* cref;   // (B) or null
  const double* pinv;   // (n,9)
  const unsigned char* frank;
  const int* inc_off;    // (n+1)
  const int* inc_split;  // (n) i-side entries of each particle
  const int2* inc;       // (2B) (bond, partner): i side ascending j, then j side ascending i
  // scratch
  double* shear;             // (n)
  double* abf;               // (B,3) active bond force (zero for a dead bond)
  unsigned long long* pkey;  // (n) packed cell of the current step
  int* pslot;                // (n) its slot in the current table, -1: not hashed
  unsigned long long* hkey;  // (2, H) two cell tables, by step parity
  int* hcnt;                 // (2, H)
  int* hfill;                // (2, H)
  int* hstart;               // (H) ranges of the current table
  int* members;              // (n)
  int* ci_cnt;    // (n)
  int* ci_j;      // (n, kContacts)
  double* ci_v;   // (n, kContacts, 9): friction force, rolling force on j, contact force
  int* ib_cnt;    // (n) inbox: pairs in which the particle is the higher id
  unsigned long long* ib_key;  // (n, kContacts) reference order key: first id of the partner's cell, partner
  int* ib_idx;    // (n, kContacts) the pair's entry in the partner's ci_v
  int* hist_cnt;  // (n) entries of each particle's history table
  int* hist_old;  // (n) entries when the step's contact phase began
  int* cellmin;   // (n) first particle of each particle's cell
  int* hist_j;    // (n, kHistory)
  double* hist_d; // (n, kHistory, 3)
  double* ledger; // TDEM_L3_COUNT
  int* status;
  unsigned hmask;
  // grid coordination
  unsigned* bar_count;
  unsigned* bar_gen;
  int* cursor;     // [2] cell-range allocation cursors, by table
  int* gflags;     // [2] status bits of the step, by step parity
  double* part;    // [grid, kPartials] per-block ledger partials
  double* pmin;    // [grid, 2] per-block min break margin, max history size
  double* pdiss;   // [grid] per-block dashpot dissipation of the launch
  unsigned long long barrier_spins;  // naps a grid barrier may wait (kBarrierSpins; tests shorten it)
};

// Grid-wide barrier of a cooperative launch. The wait is bounded: when it
// runs out the block records kStatusBarrier and the caller returns.
__device__ __noinline__ bool grid_sync(const Dev& D) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* gen = D.bar_gen;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(D.bar_count, 1u) == gridDim.x - 1) {
      atomicExch(D.bar_count, 0u);
      __threadfence();
      atomicAdd(D.bar_gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g) {
        if (++spins > D.barrier_spins) {
          ok = 0;
          atomicOr(D.status, kStatusBarrier);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

#define TDEM_GRID_SYNC() \
  do {                    \
    if (!grid_sync(D)) return; \
  } while (0)

// torch.linalg.vector_norm of a 3-vector on the CPU: one fused multiply-add
// per component after the first square, then the square root.
__device__ __forceinline__ double norm3(double x, double y, double z) { return sqrt(fma(z, z, fma(y, y, x * x))); }

__device__ __forceinline__ unsigned hash_slot(unsigned long long key, unsigned mask) {
  unsigned long long z = key * 0x9E3779B97F4A7C15ull;
  z ^= z >> 31;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 29;
  return (unsigned)z & mask;
}

__device__ __forceinline__ unsigned long long pack_cell(long long cx, long long cy, long long cz) {
  return ((unsigned long long)(cx + kCoordHalf) << 42) | ((unsigned long long)(cy + kCoordHalf) << 21) |
         (unsigned long long)(cz + kCoordHalf);
}

__device__ __forceinline__ int find_cell(const unsigned long long* hkey, unsigned mask, unsigned long long key) {
  unsigned s = hash_slot(key, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const unsigned long long k = hkey[s];
    if (k == key) return (int)s;
    if (k == kEmpty) return -1;
    s = (s + 1) & mask;
  }
  return -1;
}

// DEM3DConfig.friction_cone_limit (dem3d.py:453-498).
__device__ __forceinline__ double cone_limit(int mode, const double* c, double ft_mag, double normal, double slip) {
  if (mode == TDEM_CONE_TANH) {
    const double blend = 0.5 * (1.0 - tanh(slip / c[2]));
    return (c[0] + c[1] * blend) * normal;
  }
  if (mode == TDEM_CONE_DUAL) {
    const double st = c[0] * normal;
    return ft_mag > st ? c[1] * normal : st;
  }
  return c[0] * normal;
}

// x ** m as torch evaluates a scalar power (its special cases 1, 2, 3).
__device__ __forceinline__ double torch_pow(double x, double m) {
  if (m == 1.0) return x;
  if (m == 2.0) return x * x;
  if (m == 3.0) return x * x * x;
  return pow(x, m);
}

// Spherical-cap submerged fraction (buoyancy_wet3d.py:134-155).
__device__ __forceinline__ double submerged(const tdem_icedem3d_config& P, double z) {
  const double r = P.radius;
  const double h = z - P.water_level;
  const double hc = fmin(fmax(h, -r), r);
  const double a = r - hc;
  double f = ((a * a) * (2.0 * r + hc)) / P.cap_denominator;
  f = fmin(fmax(f, 0.0), 1.0);
  if (h >= r) f = 0.0;
  if (h <= -r) f = 1.0;
  return f;
}

// Cell of particle k at position (x, y, z) into table t (dem3d.py:836-840).
__device__ __forceinline__ void insert_cell(const Dev& D, int t, int k, double x, double y, double z, double width,
                                            int& flags) {
  const size_t H = (size_t)D.hmask + 1;
  const double fx = floor(x / width), fy = floor(y / width), fz = floor(z / width);
  const double lim = (double)kCoordHalf - 2.0;
  int slot = -1;
  if (fabs(fx) < lim && fabs(fy) < lim && fabs(fz) < lim) {
    const unsigned long long key = pack_cell((long long)fx, (long long)fy, (long long)fz);
    unsigned long long* hkey = D.hkey + t * H;
    unsigned s = hash_slot(key, D.hmask);
    for (unsigned probe = 0; probe <= D.hmask; ++probe) {
      const unsigned long long prev = atomicCAS(&hkey[s], kEmpty, key);
      if (prev == kEmpty || prev == key) {
        slot = (int)s;
        break;
      }
      s = (s + 1) & D.hmask;
    }
    if (slot >= 0) {  // always: the table has at least 2n slots
      D.pkey[k] = key;
      atomicAdd(&D.hcnt[t * H + slot], 1);
    }
  } else {
    flags |= (fx == fx && fy == fy && fz == fz) ? kStatusEscaped : kStatusNonfinite;
  }
  D.pslot[k] = slot;
}

constexpr double kTiny = 2.2250738585072014e-308;  // smallest normal double

// Mindlin-Deresiewicz partial-slip force magnitude
// mu F_n [1 - (1 - delta / delta_s)^(3/2)], delta_s = 3 mu F_n / (2 k_t)
// (mindlin_partial_slip.py:155-198).
__device__ __forceinline__ double partial_slip_mag(double delta, double fn, double mu, double kt) {
  delta = fmax(delta, 0.0);
  fn = fmax(fn, 0.0);
  const double ds = ((3.0 * mu) * fn) / (2.0 * fmax(kt, kTiny));
  const double cap = mu * fn;
  double ratio = ds > 0.0 ? delta / fmax(ds, kTiny) : 1.0;
  ratio = fmin(fmax(ratio, 0.0), 1.0);
  return cap * (1.0 - pow(fmax(1.0 - ratio, 0.0), 1.5));
}

// Platen Coulomb friction force for the spring offset t and normal force mag
// (dem3d.py:1187-1240): the Cundall-Strack spring capped by the cone, or the
// Mindlin-Deresiewicz law with k_t = 8 G* a of the rigid counterpart.
__device__ __forceinline__ void platen_friction_force(const tdem_icedem3d_config& P, const double* t, double mag,
                                                double slip, double* out) {
  if (P.mindlin) {
    const double fn = fmax(mag, 0.0);
    const double a = pow(fmax(((3.0 * fn) * P.rigid_radius) / P.rigid_4e, 0.0), 1.0 / 3.0);
    const double dm = norm3(t[0], t[1], t[2]);
    const double fm = -partial_slip_mag(dm, mag, P.platen_cone_c[0], P.mindlin_platen_8g * a);
    const double dd = fmax(dm, kEps);
    out[0] = fm * (t[0] / dd);
    out[1] = fm * (t[1] / dd);
    out[2] = fm * (t[2] / dd);
    return;
  }
  const double kk = -P.platen_kt;
  const double sx = kk * t[0], sy = kk * t[1], sz = kk * t[2];
  const double sm = norm3(sx, sy, sz);
  const double lim = cone_limit(P.platen_cone, P.platen_cone_c, sm, mag, slip);
  const double sc = sm > lim ? lim / fmax(sm, kEps) : 1.0;
  out[0] = sx * sc;
  out[1] = sy * sc;
  out[2] = sz * sc;
}

struct Out {
  double* force;      // (n,3) or null
  int mode;           // 0: steps; 1: one evaluation
  int uf, uh;         // update_fracture, update_history
  long long n_steps;
  double time;
  int mapping;        // 0: by size; 1: lanes per particle; 2: one thread per particle
};

constexpr int kChunk = 8;  // incidence entries whose loads are in flight together

__global__ void __launch_bounds__(kBlock, 1) icedem3d_kernel(tdem_icedem3d_config P, Dev D, tdem_icedem3d_state S,
                                                           const double* __restrict__ loads, Out O) {
  __shared__ double red[kPartials * (kBlock / 32)];
  const int n = P.n, nb = P.nbond;
  const int tid = threadIdx.x;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int M = P.n_branches;
  const double two_r = 2.0 * P.radius;
  const double width = 2.0 * P.radius;
  const bool friction = P.cone != TDEM_CONE_OFF;
  const bool platen_friction = P.platen_cone != TDEM_CONE_OFF;
  const size_t H = (size_t)D.hmask + 1;
  // small instances: several lanes per particle (a 16-lane group fits every
  // particle); large ones: one thread per particle, as lanes would only add
  // idle and repeated FP64 work
  const bool wide = O.mapping == 1 || (O.mapping == 0 && (long long)n * 16 <= (long long)gs);
  double* pos = S.positions;
  double* vel = S.velocities;
  double time = O.time;
  double min_margin = 1e300;
  int hist_max = 0;
  long long done = 0;
  double diss_launch = 0.0;  // this thread's dashpot dissipation over the launch
  const long long total = O.mode == 1 ? 1 : O.n_steps;

  // prologue: cells of the starting positions into table 0 (both tables
  // start cleared by the host)
  {
    int flags = 0;
    for (int k = gt; k < n; k += gs) insert_cell(D, 0, k, pos[3 * k], pos[3 * k + 1], pos[3 * k + 2], width, flags);
    if (flags) atomicOr(&D.gflags[0], flags);
  }
  TDEM_GRID_SYNC();

  for (long long step = 0; step < total; ++step) {
    const int uf = O.mode == 1 ? O.uf : 1;
    const int uh = O.mode == 1 ? O.uh : 1;
    const int p = (int)(step & 1), q = p ^ 1;  // this step's cell table, the next step's
    int flags = 0;
    // ---- A: cell ranges of table p; table q cleared; shear strain (dem3d.py:875-901)
    for (unsigned s = gt; s <= D.hmask; s += gs) {
      const int c = D.hcnt[p * H + s];
      if (c) D.hstart[s] = atomicAdd(&D.cursor[p], c);
      D.hkey[q * H + s] = kEmpty;
      D.hcnt[q * H + s] = 0;
      D.hfill[q * H + s] = 0;
    }
    if (gt == 0) D.cursor[q] = 0;
    for (int k = gt; k < n; k += gs) D.ib_cnt[k] = 0;
    if (uf && nb > 0 && wide) {
      // a 16-lane group per particle; lane w < 9 sums component w = (a, b) of
      // sum_e q_a r_b over the bond list in order (each component's sum is
      // the reference's, in its order); the group leader finishes the strain
      const int sub = threadIdx.x & 15, a = sub / 3, b = sub % 3;
      const bool comp = sub < 9;
      const int ngroups = gs >> 4;
      for (int kb = (gt >> 5) << 1; kb < n; kb += ngroups) {  // warp-uniform: two particles per warp
        const int k = kb + ((threadIdx.x >> 4) & 1);
        double c = 0.0;
        if (k < n && comp) {
          const double pka = pos[3 * k + a];
          const int e0 = D.inc_off[k], es = e0 + D.inc_split[k], e1 = D.inc_off[k + 1];
          for (int e = e0; e < e1; e += kChunk) {
            int2 ent[kChunk];
            double oa[kChunk], rb[kChunk];
#pragma unroll
            for (int w = 0; w < kChunk; ++w) ent[w] = e + w < e1 ? D.inc[e + w] : make_int2(0, k);
#pragma unroll
            for (int w = 0; w < kChunk; ++w) {
              oa[w] = pos[3 * ent[w].y + a];
              rb[w] = D.ref[3 * ent[w].x + b];
            }
#pragma unroll
            for (int w = 0; w < kChunk; ++w) {
              if (e + w >= e1) break;
              // q = x[j] - x[i] of the bond; this particle is i on its first es - e0 entries
              const double qa = e + w < es ? oa[w] - pka : pka - oa[w];
              c += qa * rb[w];
            }
          }
        }
        double cc[9];
#pragma unroll
        for (int w = 0; w < 9; ++w) cc[w] = __shfl_sync(0xffffffffu, c, w, 16);
        if (k < n && sub == 0) {
          double shear = 0.0;
          if (D.frank[k]) {
            const double* pi = D.pinv + 9 * (size_t)k;
            double f[9];
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
              for (int y = 0; y < 3; ++y)
                f[3 * x + y] = (cc[3 * x] * pi[y] + cc[3 * x + 1] * pi[3 + y]) + cc[3 * x + 2] * pi[6 + y];
            double e[9];
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
              for (int y = 0; y < 3; ++y) {
                const double g = (f[x] * f[y] + f[3 + x] * f[3 + y]) + f[6 + x] * f[6 + y];
                e[3 * x + y] = 0.5 * (g - (x == y ? 1.0 : 0.0));
              }
            const double mean = ((e[0] + e[4]) + e[8]) / 3.0;
            e[0] = e[0] - mean;
            e[4] = e[4] - mean;
            e[8] = e[8] - mean;
            // dev.square().sum(dim=(1, 2)): torch's contiguous inner sum of 9
            // values: the tail element, then the four lanes of two 4-wide loads
            double sq[9];
#pragma unroll
            for (int w = 0; w < 9; ++w) sq[w] = e[w] * e[w];
            double s2 = sq[8];
#pragma unroll
            for (int w = 0; w < 4; ++w) s2 = s2 + (sq[w] + sq[w + 4]);
            shear = sqrt((2.0 / 3.0) * fmax(s2, 0.0));
          }
          D.shear[k] = shear;
        }
      }
    } else if (uf && nb > 0) {
      // one thread per particle, its bond list fetched in chunks of loads in flight
      for (int k = gt; k < n; k += gs) {
        double c[9];
#pragma unroll
        for (int w = 0; w < 9; ++w) c[w] = 0.0;
        const double pkx = pos[3 * k], pky = pos[3 * k + 1], pkz = pos[3 * k + 2];
        const int e0 = D.inc_off[k], es = e0 + D.inc_split[k], e1 = D.inc_off[k + 1];
        for (int e = e0; e < e1; e += kChunk) {
          int2 ent[kChunk];
          double ox[kChunk], oy[kChunk], oz[kChunk], rx[kChunk], ry[kChunk], rz[kChunk];
#pragma unroll
          for (int w = 0; w < kChunk; ++w) ent[w] = e + w < e1 ? D.inc[e + w] : make_int2(0, k);
#pragma unroll
          for (int w = 0; w < kChunk; ++w) {
            const int o = ent[w].y, b = ent[w].x;
            ox[w] = pos[3 * o];
            oy[w] = pos[3 * o + 1];
            oz[w] = pos[3 * o + 2];
            rx[w] = D.ref[3 * b];
            ry[w] = D.ref[3 * b + 1];
            rz[w] = D.ref[3 * b + 2];
          }
#pragma unroll
          for (int w = 0; w < kChunk; ++w) {
            if (e + w >= e1) break;
            // q = x[j] - x[i] of the bond; this particle is i on its first es - e0 entries
            const bool iside = e + w < es;
            const double qx = iside ? ox[w] - pkx : pkx - ox[w];
            const double qy = iside ? oy[w] - pky : pky - oy[w];
            const double qz = iside ? oz[w] - pkz : pkz - oz[w];
            c[0] += qx * rx[w]; c[1] += qx * ry[w]; c[2] += qx * rz[w];
            c[3] += qy * rx[w]; c[4] += qy * ry[w]; c[5] += qy * rz[w];
            c[6] += qz * rx[w]; c[7] += qz * ry[w]; c[8] += qz * rz[w];
          }
        }
        double shear = 0.0;
        if (D.frank[k]) {
          const double* pi = D.pinv + 9 * (size_t)k;
          double f[9];
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
              f[3 * a + b] = (c[3 * a] * pi[b] + c[3 * a + 1] * pi[3 + b]) + c[3 * a + 2] * pi[6 + b];
          double e[9];
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              const double g = (f[a] * f[b] + f[3 + a] * f[3 + b]) + f[6 + a] * f[6 + b];
              e[3 * a + b] = 0.5 * (g - (a == b ? 1.0 : 0.0));
            }
          const double mean = ((e[0] + e[4]) + e[8]) / 3.0;
          e[0] = e[0] - mean;
          e[4] = e[4] - mean;
          e[8] = e[8] - mean;
          // dev.square().sum(dim=(1, 2)): torch's contiguous inner sum of 9
          // values: the tail element, then the four lanes of two 4-wide loads
          double sq[9];
#pragma unroll
          for (int w = 0; w < 9; ++w) sq[w] = e[w] * e[w];
          double s2 = sq[8];
#pragma unroll
          for (int w = 0; w < 4; ++w) s2 = s2 + (sq[w] + sq[w + 4]);
          shear = sqrt((2.0 / 3.0) * fmax(s2, 0.0));
        }
        D.shear[k] = shear;
      }
    }
    TDEM_GRID_SYNC();
    // every block has read the flags of the previous step (before the barrier
    // above), so the other parity can be cleared for the next step
    if (gt == 0) D.gflags[(step + 1) & 1] = 0;

    // ---- B: bonds: force, break commit, Maxwell branches, creep (dem3d.py:1018-1100, 1342-1360)
    for (int b = gt; b < nb; b += gs) {
      const int i = D.bi[b], j = D.bj[b];
      const double dx = pos[3 * j] - pos[3 * i];
      const double dy = pos[3 * j + 1] - pos[3 * i + 1];
      const double dz = pos[3 * j + 2] - pos[3 * i + 2];
      const double dist = norm3(dx, dy, dz);
      double nx, ny, nz;
      if (dist > kEps) {
        const double dc = fmax(dist, kEps);
        nx = dx / dc;
        ny = dy / dc;
        nz = dz / dc;
      } else {
        nx = D.inorm[3 * b];
        ny = D.inorm[3 * b + 1];
        nz = D.inorm[3 * b + 2];
      }
      const double ext = dist - D.rest[b];
      bool alive = S.alive[b] != 0;
      double mag;
      if (M == 0) {
        mag = P.bond_k * ext;
      } else {
        double* off = S.branch_offsets + (size_t)b * M;
        if (uh) {
          // advance_branches (ice_bond_viscoelastic.py:186-253), exact over the increment
          const double d_old = S.elongation_prev[b];
          const double d_dot = (ext - d_old) / P.dt;
          double dis = 0.0;
          for (int a = 0; a < M; ++a) {
            const double tau = P.branch_tau[a];
            const double s0 = d_old - off[a];
            const double amp = d_dot * tau;
            const double om = P.branch_one_minus[a], dec = P.branch_decay[a];
            const double s_new = amp * om + s0 * dec;
            const double sa = s0 - amp;
            const double i2 = ((amp * amp) * P.dt + (((2.0 * amp) * sa) * tau) * om) +
                              ((0.5 * (sa * sa)) * tau) * (om * (1.0 + dec));
            dis = dis + (P.branch_k[a] / tau) * i2;
            off[a] = alive ? ext - s_new : ext;
          }
          if (alive) diss_launch += dis;
          S.elongation_prev[b] = ext;
        }
        mag = P.bond_k * ext;
        for (int a = 0; a < M; ++a) mag = mag + P.branch_k[a] * (ext - off[a]);
      }
      if (uf && alive) {
        const double strain = ext / D.rest[b];
        const double sb = 0.5 * (D.shear[i] + D.shear[j]);
        const double thr = D.thr ? D.thr[b] : P.breaking_strain;
        const bool tf = strain > thr;
        const bool sf = sb > P.shear_breaking_strain;
        int mode = 0;
        if (tf || sf) {
          mode = (tf ? 1 : 0) + 2 * (sf ? 1 : 0);
        } else {
          min_margin = fmin(min_margin, fmin((thr - strain) / thr,
                                             (P.shear_breaking_strain - sb) / P.shear_breaking_strain));
          if (P.creep) {
            // Kachanov clock (ice_bond_viscoelastic.py:284-297, dem3d.py:1079-1100)
            const double ratio = fabs(mag) / fmax(D.cref[b], 1e-30);
            const double dmg = S.damage[b] + torch_pow(ratio, P.creep_exponent) * P.creep_dt_over_time;
            S.damage[b] = dmg;
            if (dmg >= 1.0) mode = 4;
          }
        }
        if (mode) {
          alive = false;
          S.alive[b] = 0;
          S.failure_mode[b] = (unsigned char)mode;
          S.failure_time_s[b] = time;
          S.failure_extension_m[b] = ext;
          double energy;
          if (M == 0) {
            energy = (0.5 * P.bond_k) * (ext * ext);
          } else {
            const double* off = S.branch_offsets + (size_t)b * M;
            energy = (0.5 * P.bond_k) * (ext * ext);
            for (int a = 0; a < M; ++a) {
              const double s = ext - off[a];
              energy = energy + (0.5 * P.branch_k[a]) * (s * s);
            }
          }
          S.failure_energy_J[b] = energy;
        }
      }
      D.abf[3 * b] = alive ? mag * nx : 0.0;
      D.abf[3 * b + 1] = alive ? mag * ny : 0.0;
      D.abf[3 * b + 2] = alive ? mag * nz : 0.0;
    }
    // ---- B: members into their cells of table p
    for (int k = gt; k < n; k += gs) {
      const int s = D.pslot[k];
      if (s >= 0) D.members[D.hstart[s] + atomicAdd(&D.hfill[p * H + s], 1)] = k;
    }
    TDEM_GRID_SYNC();

    const unsigned long long* hkey_p = D.hkey + p * H;
    const int* hcnt_p = D.hcnt + p * H;
    double acc_fp = 0.0, acc_rp = 0.0, acc_en = 0.0, acc_nc = 0.0;
    if (wide) {
      // ---- C1: contact candidates (dem3d.py:825-856, 1374-1381). A warp per
      // particle, lane o < 27 owning neighbour cell o in the reference's offset
      // order (dx, then dy, then dz); each lane finds its cell's overlapping
      // members with higher ids, ascending, and an exclusive prefix over the
      // lanes lays them out in the reference's pair-list order.
      {
        const int lane = threadIdx.x & 31;
        const int o = lane < 27 ? lane : 13;  // lanes 27..31 idle (13 is the own cell)
        const int dx = o / 9 - 1, dy = (o / 3) % 3 - 1, dz = o % 3 - 1;
        for (int k = gt >> 5; k < n; k += gs >> 5) {  // warp-uniform
          const int sk = D.pslot[k];
          if (lane == 0 && friction) D.hist_old[k] = min(D.hist_cnt[k], kHistory);
          int sl = -1, cnt = 0, st = 0;
          double pkx = 0.0, pky = 0.0, pkz = 0.0;
          if (sk >= 0) {
            const unsigned long long kk = D.pkey[k];
            const long long cx = (long long)(kk >> 42) - kCoordHalf;
            const long long cy = (long long)((kk >> 21) & ((1ull << 21) - 1)) - kCoordHalf;
            const long long cz = (long long)(kk & ((1ull << 21) - 1)) - kCoordHalf;
            pkx = pos[3 * k];
            pky = pos[3 * k + 1];
            pkz = pos[3 * k + 2];
            if (lane < 27) {
              sl = find_cell(hkey_p, D.hmask, pack_cell(cx + dx, cy + dy, cz + dz));
              if (sl >= 0) {
                cnt = hcnt_p[sl];
                st = D.hstart[sl];
              }
            }
          }
          // own cell's first particle (the inbox order key of this particle's pairs)
          if (lane == 13 && sk >= 0) {
            int own_min = k;
            for (int m = st; m < st + cnt; ++m) own_min = min(own_min, D.members[m]);
            D.cellmin[k] = own_min;
          }
          // pass 1: count, pass 2: write at the prefix offset
          int near = 0;
          for (int pass = 0; pass < 2; ++pass) {
            int base = 0;
            if (pass == 1) {
              int incl = near;
#pragma unroll
              for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
              }
              base = incl - near;
              const int total = __shfl_sync(0xffffffffu, incl, 31);
              if (lane == 0) D.ci_cnt[k] = min(total, kContacts);
              if (total > kContacts && lane == 0) flags |= kStatusContacts;
              if (near == 0) continue;
            }
            int w = 0, last = -1;
            for (int t = 0; t < cnt; ++t) {
              int j = INT_MAX;
              for (int m = st; m < st + cnt; ++m) {
                const int x = D.members[m];
                if (x > last && x < j) j = x;
              }
              last = j;
              if (j <= k) continue;
              const double ex = pos[3 * j] - pkx, ey = pos[3 * j + 1] - pky, ez = pos[3 * j + 2] - pkz;
              const double ov = fmax(two_r - norm3(ex, ey, ez), 0.0);
              if (!(ov > 0.0)) continue;
              if (pass == 0) {
                ++near;
              } else {
                if (base + w < kContacts) D.ci_j[(size_t)k * kContacts + base + w] = j;
                ++w;
              }
            }
          }
        }
      }
      TDEM_GRID_SYNC();
      // ---- C2: one thread per overlapping pair (dem3d.py:1382-1514): normal
      // force, friction with the pair's history, rolling couple; the partner
      // gets the pair in its inbox with the reference's order key of its side.
      for (long long tt = gt; tt < (long long)n * kContacts; tt += gs) {
        const int k = (int)(tt / kContacts), c = (int)(tt % kContacts);
        if (c >= D.ci_cnt[k]) continue;
        const int j = D.ci_j[(size_t)k * kContacts + c];
        const double pkx = pos[3 * k], pky = pos[3 * k + 1], pkz = pos[3 * k + 2];
        const double vkx = vel[3 * k], vky = vel[3 * k + 1], vkz = vel[3 * k + 2];
        const bool fk = S.fixed[k] != 0;
        const int ib0 = D.inc_off[k], ib1 = ib0 + D.inc_split[k];
        int* hj = D.hist_j + (size_t)k * kHistory;
        double* hd = D.hist_d + (size_t)k * kHistory * 3;
        const int hc = friction ? D.hist_old[k] : 0;
        const double ex = pos[3 * j] - pkx, ey = pos[3 * j + 1] - pky, ez = pos[3 * j + 2] - pkz;
        const double dist = norm3(ex, ey, ez);
        const double ov = fmax(two_r - dist, 0.0);
        acc_nc += 1.0;
                bool balive = false;
                for (int e = ib0; e < ib1; ++e) {
                  const int2 en = D.inc[e];
                  if (en.y == j) {
                    balive = S.alive[en.x] != 0;
                    break;
                  }
                }
                const double dc = fmax(dist, kEps);
                const double nx = ex / dc, ny = ey / dc, nz = ez / dc;
                const double vjx = vel[3 * j], vjy = vel[3 * j + 1], vjz = vel[3 * j + 2];
                const double rvx = vjx - vkx, rvy = vjy - vky, rvz = vjz - vkz;
                const double vn = (rvx * nx + rvy * ny) + rvz * nz;
                const bool pinned = P.any_fixed && (fk != (S.fixed[j] != 0));
                const double k_local = P.hertz ? P.hertz_kn * sqrt(ov) : P.contact_k;
                double gamma = 0.0;
                if (P.damping == 2) {
                  gamma = P.damping_c;
                } else if (P.damping == 1) {
                  gamma = P.hertz ? P.damping_c * sqrt(k_local * (pinned ? P.mass_pinned : P.mass_mobile))
                                : (pinned ? P.gamma_pinned : P.gamma_mobile);
                }
                double mag = fmax(k_local * ov - gamma * vn, 0.0);
                if (balive) mag = 0.0;
                else acc_en += P.hertz ? P.hertz_pot * pow(ov, 2.5) : (0.5 * P.contact_k) * (ov * ov);
                double* out = D.ci_v + ((size_t)k * kContacts + c) * 9;
                const double vtx = rvx - vn * nx, vty = rvy - vn * ny, vtz = rvz - vn * nz;
                if (friction) {
                  // Cundall-Strack spring with the pair's stored displacement
                  int h = -1;
                  for (int q = 0; q < hc; ++q)  // the entries that existed when the step began
                    if (hj[q] == j) {
                      h = q;
                      break;
                    }
                  double tx = 0.0, ty = 0.0, tz = 0.0;
                  if (h >= 0) {
                    tx = hd[3 * h];
                    ty = hd[3 * h + 1];
                    tz = hd[3 * h + 2];
                  }
                  if (uh) {
                    tx = tx + vtx * P.dt;
                    ty = ty + vty * P.dt;
                    tz = tz + vtz * P.dt;
                  }
                  const double kt = P.hertz_tangential ? P.hertz_kt * sqrt(ov) : P.tangential_k;
                  double Fx, Fy, Fz;
                  if (P.mindlin) {
                    // Mindlin-Deresiewicz along the displacement (mindlin_partial_slip.py:201-232)
                    const double dm = norm3(tx, ty, tz);
                    const double fmag = partial_slip_mag(dm, mag, P.cone_c[0], kt);
                    double ux = 0.0, uy = 0.0, uz = 0.0;
                    if (dm > 0.0) {
                      const double dd = fmax(dm, kTiny);
                      ux = tx / dd;
                      uy = ty / dd;
                      uz = tz / dd;
                    }
                    Fx = fmag * ux;
                    Fy = fmag * uy;
                    Fz = fmag * uz;
                  } else {
                    const double fx = kt * tx, fy = kt * ty, fz = kt * tz;
                    const double fm = norm3(fx, fy, fz);
                    const double lim = cone_limit(P.cone, P.cone_c, fm, mag, norm3(vtx, vty, vtz));
                    const double sc = fm > lim ? lim / fmax(fm, 1e-15) : 1.0;
                    Fx = fx * sc;
                    Fy = fy * sc;
                    Fz = fz * sc;
                  }
                  out[0] = Fx;
                  out[1] = Fy;
                  out[2] = Fz;
                  acc_fp += (Fx * (vkx - vjx) + Fy * (vky - vjy)) + Fz * (vkz - vjz);
                  if (uh) {
                    // the state: the displacement itself (Mindlin) or the cone projection F_t / k_t
                    const double sx = P.mindlin ? tx : Fx / kt, sy = P.mindlin ? ty : Fy / kt,
                                 sz = P.mindlin ? tz : Fz / kt;
                    if (h >= 0) {
                      hd[3 * h] = sx;
                      hd[3 * h + 1] = sy;
                      hd[3 * h + 2] = sz;
                    } else if (sx != 0.0 || sy != 0.0 || sz != 0.0) {
                      // an absent entry reads as zero, so only non-zero values need a slot
                      const int slot = atomicAdd(&D.hist_cnt[k], 1);
                      if (slot >= kHistory) {
                        flags |= kStatusHistory;
                      } else {
                        hj[slot] = j;
                        hd[3 * slot] = sx;
                        hd[3 * slot + 1] = sy;
                        hd[3 * slot + 2] = sz;
                      }
                    }
                  }
                }
                if (P.rolling) {
                  // rolling-resistance couple (dem3d.py:1242-1299)
                  const double vtm = norm3(vtx, vty, vtz);
                  double hx = 0.0, hy = 0.0, hz = 0.0;
                  if (vtm > 1e-15) {
                    const double vc = fmax(vtm, kEps);
                    hx = vtx / vc;
                    hy = vty / vc;
                    hz = vtz / vc;
                  }
                  const double fm = -(P.roll_mu * mag);
                  const double jx = fm * hx, jy = fm * hy, jz = fm * hz;
                  out[3] = jx;
                  out[4] = jy;
                  out[5] = jz;
                  acc_rp += ((-jx) * (vkx - vjx) + (-jy) * (vky - vjy)) + (-jz) * (vkz - vjz);
                }
                const double cm = -mag;
                out[6] = cm * nx;
                out[7] = cm * ny;
                out[8] = cm * nz;
        const int slot = atomicAdd(&D.ib_cnt[j], 1);
        if (slot < kContacts) {
          D.ib_key[(size_t)j * kContacts + slot] = ((unsigned long long)D.cellmin[k] << 32) | (unsigned)k;
          D.ib_idx[(size_t)j * kContacts + slot] = k * kContacts + c;
        } else {
          flags |= kStatusContacts;
        }
      }
    } else {
      // ---- C: contacts (dem3d.py:1374-1514). Each particle evaluates its pairs
      // with higher ids, over the 27 neighbour cells in the reference's order
      // and each cell's members ascending; the higher id gets the pair in its inbox.
      for (int k = gt; k < n; k += gs) {
        int nci = 0;
        const int sk = D.pslot[k];
        if (sk >= 0) {
          const unsigned long long kk = D.pkey[k];
          const long long cx = (long long)(kk >> 42) - kCoordHalf;
          const long long cy = (long long)((kk >> 21) & ((1ull << 21) - 1)) - kCoordHalf;
          const long long cz = (long long)(kk & ((1ull << 21) - 1)) - kCoordHalf;
          const double pkx = pos[3 * k], pky = pos[3 * k + 1], pkz = pos[3 * k + 2];
          const double vkx = vel[3 * k], vky = vel[3 * k + 1], vkz = vel[3 * k + 2];
          const bool fk = S.fixed[k] != 0;
          int* hj = D.hist_j + (size_t)k * kHistory;
          double* hd = D.hist_d + (size_t)k * kHistory * 3;
          int hc = friction ? D.hist_cnt[k] : 0;
          const int ib0 = D.inc_off[k], ib1 = ib0 + D.inc_split[k];
          // the first particle of this particle's cell orders the pair in the partner's inbox
          int own_min = k;
          {
            const int m0 = D.hstart[sk], m1 = m0 + hcnt_p[sk];
            for (int m = m0; m < m1; ++m) own_min = min(own_min, D.members[m]);
          }
          const unsigned long long own_key = (unsigned long long)own_min << 32;
          for (int dx = -1; dx <= 1; ++dx) {
            // the nine cells of this dx: lookups, then counts and starts, in flight together
            int sl[9], cnt[9], st[9];
            unsigned long long ck[9], first[9];
            unsigned hs[9];
  #pragma unroll
            for (int o = 0; o < 9; ++o) {
              ck[o] = pack_cell(cx + dx, cy + o / 3 - 1, cz + o % 3 - 1);
              hs[o] = hash_slot(ck[o], D.hmask);
              first[o] = hkey_p[hs[o]];
            }
  #pragma unroll
            for (int o = 0; o < 9; ++o)  // a collision probes on (rare)
              sl[o] = first[o] == ck[o] ? (int)hs[o] : (first[o] == kEmpty ? -1 : find_cell(hkey_p, D.hmask, ck[o]));
  #pragma unroll
            for (int o = 0; o < 9; ++o) {
              cnt[o] = sl[o] >= 0 ? hcnt_p[sl[o]] : 0;
              st[o] = sl[o] >= 0 ? D.hstart[sl[o]] : 0;
            }
            for (int o = 0; o < 9; ++o) {
              // members of the cell ascending: repeated selection (cells hold a few)
              int last = -1;
              for (int t = 0; t < cnt[o]; ++t) {
                int j = INT_MAX;
                for (int m = st[o]; m < st[o] + cnt[o]; ++m) {
                  const int x = D.members[m];
                  if (x > last && x < j) j = x;
                }
                last = j;
                if (j <= k) continue;
                const double ex = pos[3 * j] - pkx, ey = pos[3 * j + 1] - pky, ez = pos[3 * j + 2] - pkz;
                const double dist = norm3(ex, ey, ez);
                const double ov = fmax(two_r - dist, 0.0);
                if (!(ov > 0.0)) continue;
                if (nci == kContacts) {
                  flags |= kStatusContacts;
                  continue;
                }
                bool balive = false;
                for (int e = ib0; e < ib1; ++e) {
                  const int2 en = D.inc[e];
                  if (en.y == j) {
                    balive = S.alive[en.x] != 0;
                    break;
                  }
                }
                const double dc = fmax(dist, kEps);
                const double nx = ex / dc, ny = ey / dc, nz = ez / dc;
                const double vjx = vel[3 * j], vjy = vel[3 * j + 1], vjz = vel[3 * j + 2];
                const double rvx = vjx - vkx, rvy = vjy - vky, rvz = vjz - vkz;
                const double vn = (rvx * nx + rvy * ny) + rvz * nz;
                const bool pinned = P.any_fixed && (fk != (S.fixed[j] != 0));
                const double k_local = P.hertz ? P.hertz_kn * sqrt(ov) : P.contact_k;
                double gamma = 0.0;
                if (P.damping == 2) {
                  gamma = P.damping_c;
                } else if (P.damping == 1) {
                  gamma = P.hertz ? P.damping_c * sqrt(k_local * (pinned ? P.mass_pinned : P.mass_mobile))
                                : (pinned ? P.gamma_pinned : P.gamma_mobile);
                }
                double mag = fmax(k_local * ov - gamma * vn, 0.0);
                if (balive) mag = 0.0;
                else acc_en += P.hertz ? P.hertz_pot * pow(ov, 2.5) : (0.5 * P.contact_k) * (ov * ov);
                double* out = D.ci_v + ((size_t)k * kContacts + nci) * 9;
                const double vtx = rvx - vn * nx, vty = rvy - vn * ny, vtz = rvz - vn * nz;
                if (friction) {
                  // Cundall-Strack spring with the pair's stored displacement
                  int h = -1;
                  for (int q = 0; q < hc; ++q)
                    if (hj[q] == j) {
                      h = q;
                      break;
                    }
                  double tx = 0.0, ty = 0.0, tz = 0.0;
                  if (h >= 0) {
                    tx = hd[3 * h];
                    ty = hd[3 * h + 1];
                    tz = hd[3 * h + 2];
                  }
                  if (uh) {
                    tx = tx + vtx * P.dt;
                    ty = ty + vty * P.dt;
                    tz = tz + vtz * P.dt;
                  }
                  const double kt = P.hertz_tangential ? P.hertz_kt * sqrt(ov) : P.tangential_k;
                  double Fx, Fy, Fz;
                  if (P.mindlin) {
                    // Mindlin-Deresiewicz along the displacement (mindlin_partial_slip.py:201-232)
                    const double dm = norm3(tx, ty, tz);
                    const double fmag = partial_slip_mag(dm, mag, P.cone_c[0], kt);
                    double ux = 0.0, uy = 0.0, uz = 0.0;
                    if (dm > 0.0) {
                      const double dd = fmax(dm, kTiny);
                      ux = tx / dd;
                      uy = ty / dd;
                      uz = tz / dd;
                    }
                    Fx = fmag * ux;
                    Fy = fmag * uy;
                    Fz = fmag * uz;
                  } else {
                    const double fx = kt * tx, fy = kt * ty, fz = kt * tz;
                    const double fm = norm3(fx, fy, fz);
                    const double lim = cone_limit(P.cone, P.cone_c, fm, mag, norm3(vtx, vty, vtz));
                    const double sc = fm > lim ? lim / fmax(fm, 1e-15) : 1.0;
                    Fx = fx * sc;
                    Fy = fy * sc;
                    Fz = fz * sc;
                  }
                  out[0] = Fx;
                  out[1] = Fy;
                  out[2] = Fz;
                  acc_fp += (Fx * (vkx - vjx) + Fy * (vky - vjy)) + Fz * (vkz - vjz);
                  if (uh) {
                    // the state: the displacement itself (Mindlin) or the cone projection F_t / k_t
                    const double sx = P.mindlin ? tx : Fx / kt, sy = P.mindlin ? ty : Fy / kt,
                                 sz = P.mindlin ? tz : Fz / kt;
                    if (h >= 0) {
                      hd[3 * h] = sx;
                      hd[3 * h + 1] = sy;
                      hd[3 * h + 2] = sz;
                    } else if (sx != 0.0 || sy != 0.0 || sz != 0.0) {
                      // an absent entry reads as zero, so only non-zero values need a slot
                      if (hc == kHistory) {
                        flags |= kStatusHistory;
                      } else {
                        hj[hc] = j;
                        hd[3 * hc] = sx;
                        hd[3 * hc + 1] = sy;
                        hd[3 * hc + 2] = sz;
                        ++hc;
                      }
                    }
                  }
                }
                if (P.rolling) {
                  // rolling-resistance couple (dem3d.py:1242-1299)
                  const double vtm = norm3(vtx, vty, vtz);
                  double hx = 0.0, hy = 0.0, hz = 0.0;
                  if (vtm > 1e-15) {
                    const double vc = fmax(vtm, kEps);
                    hx = vtx / vc;
                    hy = vty / vc;
                    hz = vtz / vc;
                  }
                  const double fm = -(P.roll_mu * mag);
                  const double jx = fm * hx, jy = fm * hy, jz = fm * hz;
                  out[3] = jx;
                  out[4] = jy;
                  out[5] = jz;
                  acc_rp += ((-jx) * (vkx - vjx) + (-jy) * (vky - vjy)) + (-jz) * (vkz - vjz);
                }
                const double cm = -mag;
                out[6] = cm * nx;
                out[7] = cm * ny;
                out[8] = cm * nz;
                D.ci_j[(size_t)k * kContacts + nci] = j;
                const int slot = atomicAdd(&D.ib_cnt[j], 1);
                if (slot < kContacts) {
                  D.ib_key[(size_t)j * kContacts + slot] = own_key | (unsigned)k;
                  D.ib_idx[(size_t)j * kContacts + slot] = k * kContacts + nci;
                } else {
                  flags |= kStatusContacts;
                }
                ++nci;
              }
            }
          }
          if (friction) {
            D.hist_cnt[k] = hc;
            hist_max = max(hist_max, hc);
          }
        }
        D.ci_cnt[k] = nci;
        acc_nc += (double)nci;
      }
    }
    TDEM_GRID_SYNC();

    // ---- D: assembly and semi-implicit Euler (dem3d.py:1326-1340, 1516-1663)
    double acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.0;
    const double tpx = P.tool_start[0] + time * P.tool_velocity[0];
    const double tpy = P.tool_start[1] + time * P.tool_velocity[1];
    const double tpz = P.tool_start[2] + time * P.tool_velocity[2];
    const double top_z = P.top_start_z + time * P.top_velocity;
    const double bottom_z = P.bottom_start_z + time * P.bottom_velocity;
    double lp[4] = {0.0, 0.0, 0.0, 0.0}, lvx = 0.0, lvy = 0.0;
    if (P.platens & 4) {
      for (int q = 0; q < 4; ++q) lp[q] = S.lateral_position[q];
      lvx = S.lateral_velocity[0];
      lvy = S.lateral_velocity[2];
    }
    if (wide) {
      const int w = threadIdx.x & 3;
      const int ngroups = gs >> 2;
      for (int kb = (gt >> 5) << 3; kb < n; kb += ngroups) {  // warp-uniform: eight particles per warp
        const int k = kb + ((threadIdx.x >> 2) & 7);
        const bool act = k < n, on = act && w < 3;
        double px = 0.0, py = 0.0, pz = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
        double tdv[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
        if (act) {
          px = pos[3 * k];
          py = pos[3 * k + 1];
          pz = pos[3 * k + 2];
          vx = vel[3 * k];
          vy = vel[3 * k + 1];
          vz = vel[3 * k + 2];
          if (platen_friction)
            for (int c = 0; c < 3; ++c) {
              tdv[0][c] = S.top_tangential[3 * (size_t)k + c];
              tdv[1][c] = S.bottom_tangential[3 * (size_t)k + c];
            }
        }
        const double pw = w == 0 ? px : (w == 1 ? py : pz);
        const double vw = w == 0 ? vx : (w == 1 ? vy : vz);
        double f = 0.0, nv = 0.0, np = 0.0;
        if (on) {
          f = (-P.drag) * vw;
          if (P.body & 1) {
            double bw = 0.0;
            if (w == 2 && P.gravity_force > 0.0) bw = bw - P.gravity_force;
            if (P.body & 2) {
              const double fs = submerged(P, pz);
              if (w == 2) bw = bw + P.buoyancy_force * fs;
              if (P.body & 4) {
                const double c = P.wet_drag * fs;
                bw = bw - c * vw;
              }
            }
            f = f + bw;
          }
          if (loads) f = f + loads[3 * k + w];
          // bonds: i side then j side in bond order, as the two index_add_ calls
          // add them (a dead bond adds its zero too)
          const int e0 = D.inc_off[k], es = e0 + D.inc_split[k], e1 = D.inc_off[k + 1];
          for (int e = e0; e < e1; e += kChunk) {
            int2 ent[kChunk];
            double aw[kChunk];
#pragma unroll
            for (int c = 0; c < kChunk; ++c) ent[c] = e + c < e1 ? D.inc[e + c] : make_int2(0, 0);
#pragma unroll
            for (int c = 0; c < kChunk; ++c) aw[c] = D.abf[3 * (size_t)ent[c].x + w];
#pragma unroll
            for (int c = 0; c < kChunk; ++c) {
              if (e + c >= e1) break;
              if (e + c < es) f += aw[c];
              else f += -aw[c];
            }
          }
          const int nci = D.ci_cnt[k];
          const double* mine = D.ci_v + (size_t)k * kContacts * 9;
          // inbox in the reference's order of the pairs in which this particle is second
          const int nib = min(D.ib_cnt[k], kContacts);
          unsigned long long ik[kContacts];
          int ix[kContacts];
          for (int a = 0; a < nib; ++a) {
            const unsigned long long key = D.ib_key[(size_t)k * kContacts + a];
            const int idx = D.ib_idx[(size_t)k * kContacts + a];
            int b = a - 1;
            while (b >= 0 && ik[b] > key) {
              ik[b + 1] = ik[b];
              ix[b + 1] = ix[b];
              --b;
            }
            ik[b + 1] = key;
            ix[b + 1] = idx;
          }
          // contact terms, in order; each chunk's loads are in flight together
          auto own_sum = [&](int off, bool neg) {
            for (int c0 = 0; c0 < nci; c0 += kChunk) {
              double val[kChunk];
#pragma unroll
              for (int c = 0; c < kChunk; ++c) val[c] = c0 + c < nci ? mine[9 * (c0 + c) + off + w] : 0.0;
#pragma unroll
              for (int c = 0; c < kChunk; ++c)
                if (c0 + c < nci) f += neg ? -val[c] : val[c];
            }
          };
          auto inbox_sum = [&](int off, bool neg) {
            for (int c0 = 0; c0 < nib; c0 += kChunk) {
              double val[kChunk];
#pragma unroll
              for (int c = 0; c < kChunk; ++c)
                val[c] = c0 + c < nib ? D.ci_v[(size_t)ix[c0 + c] * 9 + off + w] : 0.0;
#pragma unroll
              for (int c = 0; c < kChunk; ++c)
                if (c0 + c < nib) f += neg ? -val[c] : val[c];
            }
          };
          if (friction) {
            own_sum(0, false);
            inbox_sum(0, true);
          }
          if (P.rolling) {
            own_sum(3, true);
            inbox_sum(3, false);
          }
          own_sum(6, false);
          inbox_sum(6, true);
          // spherical indenter (dem3d.py:1519-1532)
          {
            const double dx = px - tpx, dy = py - tpy, dz = pz - tpz;
            const double dist = norm3(dx, dy, dz);
            double nx = 0.0, ny = 0.0, nz = -1.0;
            if (dist > kEps) {
              const double dc = fmax(dist, kEps);
              nx = dx / dc;
              ny = dy / dc;
              nz = dz / dc;
            }
            const double ov = fmax((P.radius + P.tool_radius) - dist, 0.0);
            const double vn = ((vx - P.tool_velocity[0]) * nx + (vy - P.tool_velocity[1]) * ny) +
                              (vz - P.tool_velocity[2]) * nz;
            const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.contact_k * ov;
            double mag = fmax(el - P.tool_damping * vn, 0.0);
            if (!(ov > 0.0)) mag = 0.0;
            const double tw = mag * (w == 0 ? nx : (w == 1 ? ny : nz));
            acc[w] += tw;
            f += tw;
          }
          // plane platens (dem3d.py:1534-1580) with Coulomb friction (dem3d.py:1187-1240)
          for (int side = 0; side < 2; ++side) {
            if (!(P.platens & (1 << side))) continue;
            double ov, mag;
            if (side == 0) {
              ov = fmax((pz + P.radius) - top_z, 0.0);
              const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.platen_k * ov;
              mag = fmax(el + P.platen_c * (vz - P.top_velocity), 0.0);
              if (!(ov > 0.0)) mag = 0.0;
              if (w == 2) {
                f += -mag;
                acc[3] += mag;
              }
            } else {
              ov = fmax((bottom_z + P.radius) - pz, 0.0);
              const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.platen_k * ov;
              mag = fmax(el - P.platen_c * (vz - P.bottom_velocity), 0.0);
              if (!(ov > 0.0)) mag = 0.0;
              if (w == 2) {
                f += mag;
                acc[4] += -mag;
              }
            }
            if (platen_friction) {
              const bool touch = ov > 0.0;
              const double ux = touch ? vx : 0.0, uy = touch ? vy : 0.0;
              const double slip = norm3(ux, uy, 0.0);
              double* t = tdv[side];
              if (uh) {
                t[0] = t[0] + ux * P.dt;
                t[1] = t[1] + uy * P.dt;
                t[2] = t[2] + 0.0 * P.dt;
                if (!touch) t[0] = t[1] = t[2] = 0.0;
              }
              double fr[3];
              platen_friction_force(P, t, mag, slip, fr);
              f += fr[w];
            }
          }
          if ((P.platens & 4) && w < 2) {
            // lateral servo platens (dem3d.py:1582-1623): lane 0 the x planes, lane 1 the y planes
            const double r = P.radius;
            const double lv = w == 0 ? lvx : lvy;
            double ov = fmax((lp[2 * w] - pw) + r, 0.0);
            double mg = fmax(P.lateral_k * ov - P.lateral_c * (vw - lv), 0.0);
            if (!(ov > 0.0)) mg = 0.0;
            f += mg;
            acc[5 + 2 * w] += -mg;
            ov = fmax((pw + r) - lp[2 * w + 1], 0.0);
            mg = fmax(P.lateral_k * ov + P.lateral_c * (vw - lv), 0.0);
            if (!(ov > 0.0)) mg = 0.0;
            f -= mg;
            acc[6 + 2 * w] += mg;
          }
          if (O.mode == 1) {
            O.force[3 * k + w] = f;
          } else {
            const bool fixed = S.fixed[k] != 0;
            double a = f / P.mass;
            if (fixed) a = 0.0;
            nv = vw + a * P.dt;
            if (fixed) nv = 0.0;
            np = pw + nv * P.dt;
            if (fixed) np = S.initial_positions[3 * k + w];
          }
        }
        __syncwarp();  // every lane has read the particle's state
        if (on && O.mode != 1) {
          vel[3 * k + w] = nv;
          pos[3 * k + w] = np;
          if (platen_friction && uh) {
            if (P.platens & 1) S.top_tangential[3 * (size_t)k + w] = tdv[0][w];
            if (P.platens & 2) S.bottom_tangential[3 * (size_t)k + w] = tdv[1][w];
          }
          if (!(isfinite(np) && isfinite(nv))) flags |= kStatusNonfinite;
        }
        const double n0 = __shfl_sync(0xffffffffu, np, 0, 4);
        const double n1 = __shfl_sync(0xffffffffu, np, 1, 4);
        const double n2 = __shfl_sync(0xffffffffu, np, 2, 4);
        if (act && w == 0) {
          if (O.mode != 1) insert_cell(D, q, k, n0, n1, n2, width, flags);  // the next step's cell table
          if (friction) hist_max = max(hist_max, min(D.hist_cnt[k], kHistory));
        }
      }
    } else {
      // one thread per particle
      for (int k = gt; k < n; k += gs) {
        const double px = pos[3 * k], py = pos[3 * k + 1], pz = pos[3 * k + 2];
        const double vx = vel[3 * k], vy = vel[3 * k + 1], vz = vel[3 * k + 2];
        double fx = (-P.drag) * vx, fy = (-P.drag) * vy, fz = (-P.drag) * vz;
        if (P.body & 1) {
          double bx = 0.0, by = 0.0, bz = 0.0;
          if (P.gravity_force > 0.0) bz = bz - P.gravity_force;
          if (P.body & 2) {
            const double fs = submerged(P, pz);
            bz = bz + P.buoyancy_force * fs;
            if (P.body & 4) {
              const double c = P.wet_drag * fs;
              bx = bx - c * vx;
              by = by - c * vy;
              bz = bz - c * vz;
            }
          }
          fx = fx + bx;
          fy = fy + by;
          fz = fz + bz;
        }
        if (loads) {
          fx = fx + loads[3 * k];
          fy = fy + loads[3 * k + 1];
          fz = fz + loads[3 * k + 2];
        }
        // bonds: i side then j side in bond order, as the two index_add_ calls
        // add them (a dead bond adds its zero too)
        const int e0 = D.inc_off[k], es = e0 + D.inc_split[k], e1 = D.inc_off[k + 1];
        for (int e = e0; e < e1; e += kChunk) {
          int2 ent[kChunk];
          double ax[kChunk], ay[kChunk], az[kChunk];
  #pragma unroll
          for (int w = 0; w < kChunk; ++w) ent[w] = e + w < e1 ? D.inc[e + w] : make_int2(0, 0);
  #pragma unroll
          for (int w = 0; w < kChunk; ++w) {
            const double* a = D.abf + 3 * (size_t)ent[w].x;
            ax[w] = a[0];
            ay[w] = a[1];
            az[w] = a[2];
          }
  #pragma unroll
          for (int w = 0; w < kChunk; ++w) {
            if (e + w >= e1) break;
            if (e + w < es) {
              fx += ax[w];
              fy += ay[w];
              fz += az[w];
            } else {
              fx += -ax[w];
              fy += -ay[w];
              fz += -az[w];
            }
          }
        }
        const int nci = D.ci_cnt[k];
        const double* mine = D.ci_v + (size_t)k * kContacts * 9;
        // inbox in the reference's order of the pairs in which this particle is second
        const int nib = min(D.ib_cnt[k], kContacts);
        unsigned long long ik[kContacts];
        int ix[kContacts];
        for (int a = 0; a < nib; ++a) {
          const unsigned long long key = D.ib_key[(size_t)k * kContacts + a];
          const int idx = D.ib_idx[(size_t)k * kContacts + a];
          int b = a - 1;
          while (b >= 0 && ik[b] > key) {
            ik[b + 1] = ik[b];
            ix[b + 1] = ix[b];
            --b;
          }
          ik[b + 1] = key;
          ix[b + 1] = idx;
        }
        if (friction) {
          for (int c = 0; c < nci; ++c) {
            fx += mine[9 * c];
            fy += mine[9 * c + 1];
            fz += mine[9 * c + 2];
          }
          for (int c = 0; c < nib; ++c) {
            const double* t = D.ci_v + (size_t)ix[c] * 9;
            fx += -t[0];
            fy += -t[1];
            fz += -t[2];
          }
        }
        if (P.rolling) {
          for (int c = 0; c < nci; ++c) {
            fx += -mine[9 * c + 3];
            fy += -mine[9 * c + 4];
            fz += -mine[9 * c + 5];
          }
          for (int c = 0; c < nib; ++c) {
            const double* t = D.ci_v + (size_t)ix[c] * 9;
            fx += t[3];
            fy += t[4];
            fz += t[5];
          }
        }
        for (int c = 0; c < nci; ++c) {
          fx += mine[9 * c + 6];
          fy += mine[9 * c + 7];
          fz += mine[9 * c + 8];
        }
        for (int c = 0; c < nib; ++c) {
          const double* t = D.ci_v + (size_t)ix[c] * 9;
          fx += -t[6];
          fy += -t[7];
          fz += -t[8];
        }
        // spherical indenter (dem3d.py:1519-1532)
        {
          const double dx = px - tpx, dy = py - tpy, dz = pz - tpz;
          const double dist = norm3(dx, dy, dz);
          double nx = 0.0, ny = 0.0, nz = -1.0;
          if (dist > kEps) {
            const double dc = fmax(dist, kEps);
            nx = dx / dc;
            ny = dy / dc;
            nz = dz / dc;
          }
          const double ov = fmax((P.radius + P.tool_radius) - dist, 0.0);
          const double vn = ((vx - P.tool_velocity[0]) * nx + (vy - P.tool_velocity[1]) * ny) +
                            (vz - P.tool_velocity[2]) * nz;
          const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.contact_k * ov;
          double mag = fmax(el - P.tool_damping * vn, 0.0);
          if (!(ov > 0.0)) mag = 0.0;
          const double tx = mag * nx, ty = mag * ny, tz = mag * nz;
          acc[0] += tx;
          acc[1] += ty;
          acc[2] += tz;
          fx += tx;
          fy += ty;
          fz += tz;
        }
        // plane platens (dem3d.py:1534-1580) with Coulomb friction (dem3d.py:1187-1240)
        for (int side = 0; side < 2; ++side) {
          if (!(P.platens & (1 << side))) continue;
          double ov, mag;
          if (side == 0) {
            ov = fmax((pz + P.radius) - top_z, 0.0);
            const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.platen_k * ov;
            mag = fmax(el + P.platen_c * (vz - P.top_velocity), 0.0);
            if (!(ov > 0.0)) mag = 0.0;
            fz += -mag;
            acc[3] += mag;
          } else {
            ov = fmax((bottom_z + P.radius) - pz, 0.0);
            const double el = P.hertz ? P.hertz_kn_rigid * pow(ov, 1.5) : P.platen_k * ov;
            mag = fmax(el - P.platen_c * (vz - P.bottom_velocity), 0.0);
            if (!(ov > 0.0)) mag = 0.0;
            fz += mag;
            acc[4] += -mag;
          }
          if (platen_friction) {
            double* td = (side == 0 ? S.top_tangential : S.bottom_tangential) + 3 * (size_t)k;
            const bool touch = ov > 0.0;
            const double ux = touch ? vx : 0.0, uy = touch ? vy : 0.0;
            const double slip = norm3(ux, uy, 0.0);
            double tx = td[0], ty = td[1], tz = td[2];
            if (uh) {
              tx = tx + ux * P.dt;
              ty = ty + uy * P.dt;
              tz = tz + 0.0 * P.dt;
              if (!touch) tx = ty = tz = 0.0;
              td[0] = tx;
              td[1] = ty;
              td[2] = tz;
            }
            const double tv[3] = {tx, ty, tz};
            double fr[3];
            platen_friction_force(P, tv, mag, slip, fr);
            fx += fr[0];
            fy += fr[1];
            fz += fr[2];
          }
        }
        if (P.platens & 4) {
          // lateral servo platens (dem3d.py:1582-1623)
          const double r = P.radius;
          double ov = fmax((lp[0] - px) + r, 0.0);
          double mg = fmax(P.lateral_k * ov - P.lateral_c * (vx - lvx), 0.0);
          if (!(ov > 0.0)) mg = 0.0;
          fx += mg;
          acc[5] += -mg;
          ov = fmax((px + r) - lp[1], 0.0);
          mg = fmax(P.lateral_k * ov + P.lateral_c * (vx - lvx), 0.0);
          if (!(ov > 0.0)) mg = 0.0;
          fx -= mg;
          acc[6] += mg;
          ov = fmax((lp[2] - py) + r, 0.0);
          mg = fmax(P.lateral_k * ov - P.lateral_c * (vy - lvy), 0.0);
          if (!(ov > 0.0)) mg = 0.0;
          fy += mg;
          acc[7] += -mg;
          ov = fmax((py + r) - lp[3], 0.0);
          mg = fmax(P.lateral_k * ov + P.lateral_c * (vy - lvy), 0.0);
          if (!(ov > 0.0)) mg = 0.0;
          fy -= mg;
          acc[8] += mg;
        }
        if (O.mode == 1) {
          O.force[3 * k] = fx;
          O.force[3 * k + 1] = fy;
          O.force[3 * k + 2] = fz;
          continue;
        }
        double ax = fx / P.mass, ay = fy / P.mass, az = fz / P.mass;
        const bool fixed = S.fixed[k] != 0;
        if (fixed) ax = ay = az = 0.0;
        double nvx = vx + ax * P.dt, nvy = vy + ay * P.dt, nvz = vz + az * P.dt;
        if (fixed) nvx = nvy = nvz = 0.0;
        double npx = px + nvx * P.dt, npy = py + nvy * P.dt, npz = pz + nvz * P.dt;
        if (fixed) {
          npx = S.initial_positions[3 * k];
          npy = S.initial_positions[3 * k + 1];
          npz = S.initial_positions[3 * k + 2];
        }
        vel[3 * k] = nvx;
        vel[3 * k + 1] = nvy;
        vel[3 * k + 2] = nvz;
        pos[3 * k] = npx;
        pos[3 * k + 1] = npy;
        pos[3 * k + 2] = npz;
        if (!(isfinite(npx) && isfinite(npy) && isfinite(npz) && isfinite(nvx) && isfinite(nvy) && isfinite(nvz)))
          flags |= kStatusNonfinite;
        insert_cell(D, q, k, npx, npy, npz, width, flags);  // the next step's cell table
      }
      if (friction)
        for (int k = gt; k < n; k += gs) hist_max = max(hist_max, min(D.hist_cnt[k], kHistory));
    }
    acc[9] = acc_fp;
    acc[10] = acc_rp;
    acc[11] = acc_en;
    acc[12] = acc_nc;
    if (flags) atomicOr(&D.gflags[step & 1], flags);
    // per-block ledger partials: only the launch's last evaluation is reported
    // (margins, history sizes and dissipation accumulate per thread meanwhile)
    auto write_partials = [&]() {
      double tot[kPartials];
      block_sum_f64<kPartials>(acc, red, tot);
      const double mm = block_min_f64(min_margin, red);
      const double hm = -block_min_f64(-(double)hist_max, red);
      double dv[1] = {diss_launch}, dtot[1];
      block_sum_f64<1>(dv, red, dtot);
      if (tid == 0) {
        for (int c = 0; c < kPartials; ++c) D.part[(size_t)blockIdx.x * kPartials + c] = tot[c];
        D.pmin[2 * blockIdx.x] = mm;
        D.pmin[2 * blockIdx.x + 1] = hm;
        D.pdiss[blockIdx.x] = dtot[0];
      }
    };
    const bool final_step = O.mode == 1 || step + 1 == total;
    if (final_step) write_partials();
    TDEM_GRID_SYNC();
    // every block takes the same exit decision: this parity's flags are final
    // after the barrier and are cleared only two steps later
    const int f = *reinterpret_cast<volatile int*>(&D.gflags[step & 1]);
    const bool last = final_step || f != 0;
    if (last && !final_step) {  // an early exit on a status: its partials too
      write_partials();
      TDEM_GRID_SYNC();
    }
    if (O.mode != 1) {
      if (blockIdx.x == 0 && (P.platens & 4) && tid < 4)
        S.lateral_position[tid] = lp[tid] + S.lateral_velocity[tid] * P.dt;
      time = time + P.dt;
    }
    done = step + 1;
    if (last) {
      if (blockIdx.x == 0 && tid < kPartials + 3) {
        // ledger of the last evaluation: per-block partials in block order
        double* L = D.ledger;
        const int q = tid;
        if (q < kPartials) {
          double s = 0.0;
          for (unsigned bk = 0; bk < gridDim.x; ++bk) s += D.part[(size_t)bk * kPartials + q];
          const double neg = -s;
          if (q < 3) L[TDEM_L3_REACTION_X + q] = neg;
          else if (q == 3) L[TDEM_L3_TOP_REACTION_Z] = s;
          else if (q == 4) L[TDEM_L3_BOTTOM_REACTION_Z] = s;
          else if (q < 9) L[TDEM_L3_LATERAL_0 + q - 5] = s;
          else if (q == 9 && uh) L[TDEM_L3_FRICTION_POWER] = s;
          else if (q == 10 && uh) L[TDEM_L3_ROLLING_POWER] = s;
          else if (q == 11) L[TDEM_L3_CONTACT_ENERGY] = s;
          else if (q == 12) L[TDEM_L3_CONTACTS] = s;
        } else if (q == kPartials) {
          double m = L[TDEM_L3_MIN_BREAK_MARGIN];
          for (unsigned bk = 0; bk < gridDim.x; ++bk) m = fmin(m, D.pmin[2 * bk]);
          L[TDEM_L3_MIN_BREAK_MARGIN] = m;
        } else if (q == kPartials + 1) {
          double m = 0.0;
          for (unsigned bk = 0; bk < gridDim.x; ++bk) m = fmax(m, D.pmin[2 * bk + 1]);
          L[TDEM_L3_HISTORY_MAX] = m;
        } else if (S.bond_dissipation && M > 0) {
          double s = 0.0;
          for (unsigned bk = 0; bk < gridDim.x; ++bk) s += D.pdiss[bk];
          S.bond_dissipation[0] = S.bond_dissipation[0] + s;
        }
      }
      if (gt == 0) {
        if (f) atomicOr(D.status, f);
        D.ledger[TDEM_L3_STEPS_DONE] = (double)done;
      }
      return;
    }
  }
}

}  // namespace icedem3d
}  // namespace tdem

using namespace tdem::icedem3d;

struct tdem_icedem3d {
  tdem_icedem3d_config cfg{};
  Dev dev{};
  int max_grid = 1;  // co-resident blocks of the cooperative launch
  int mapping = 0;   // TDEM_ICE3D_MAP_*
  std::vector<void*> allocs;
  double* ledger_host = nullptr;
  int* status_host = nullptr;
  std::string err;
  int n = 0, nb = 0;
};

namespace {

std::string g_create_error3;

template <class T>
int dalloc(tdem_icedem3d* h, T** p, size_t count) {
  void* q = nullptr;
  TDEM_CUDA_TRY(&h->err, cudaMalloc(&q, std::max<size_t>(1, count) * sizeof(T)));
  h->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return TDEM_OK;
}

template <class T>
int dupload(tdem_icedem3d* h, const T** dst, const T* src, size_t count) {
  T* p = nullptr;
  int rc = dalloc(h, &p, count);
  if (rc) return rc;
  if (count) TDEM_CUDA_TRY(&h->err, cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
  *dst = p;
  return TDEM_OK;
}

void destroy(tdem_icedem3d* h) {
  if (!h) return;
  for (void* p : h->allocs) cudaFree(p);
  if (h->ledger_host) cudaFreeHost(h->ledger_host);
  if (h->status_host) cudaFreeHost(h->status_host);
  delete h;
}

int check_state(tdem_icedem3d* h, const tdem_icedem3d_state* st) {
  const tdem_icedem3d_config& c = h->cfg;
  if (!st || !st->positions || !st->velocities || !st->initial_positions || !st->fixed)
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "state needs positions, velocities, initial positions and fixed");
  if (h->nb > 0 && (!st->alive || !st->failure_mode || !st->failure_time_s || !st->failure_extension_m ||
                    !st->failure_energy_J))
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "state needs the bond arrays");
  if (c.n_branches > 0 && (!st->branch_offsets || !st->elongation_prev))
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "Maxwell bonds need branch offsets and elongations");
  if (c.creep && !st->damage) return tdem::fail(&h->err, TDEM_ERR_BADARG, "creep needs the damage array");
  if (c.platen_cone != TDEM_CONE_OFF && (!st->top_tangential || !st->bottom_tangential))
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "platen friction needs the platen spring offsets");
  if ((c.platens & 4) && (!st->lateral_position || !st->lateral_velocity))
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "lateral platens need their positions and velocities");
  return TDEM_OK;
}

int launch(tdem_icedem3d* h, const tdem_icedem3d_state* st, const double* loads, Out o, cudaStream_t s) {
  int rc = check_state(h, st);
  if (rc) return rc;
  Dev& D = h->dev;
  const size_t H = (size_t)D.hmask + 1;
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.status, 0, sizeof(int), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.bar_count, 0, sizeof(unsigned), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.gflags, 0, 2 * sizeof(int), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.hkey, 0xff, 2 * H * sizeof(unsigned long long), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.hcnt, 0, 2 * H * sizeof(int), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.hfill, 0, 2 * H * sizeof(int), s));
  TDEM_CUDA_TRY(&h->err, cudaMemsetAsync(D.cursor, 0, 2 * sizeof(int), s));
  const long long items = std::max<long long>(h->n, h->nb);
  const int grid = (int)std::max<long long>(1, std::min<long long>(h->max_grid, (items + kItemsPerBlock - 1) /
                                                                                  kItemsPerBlock));
  tdem_icedem3d_config cfg = h->cfg;
  tdem_icedem3d_state state = *st;
  void* args[] = {&cfg, &D, &state, const_cast<double**>(&loads), &o};
  TDEM_CUDA_TRY(&h->err, cudaLaunchCooperativeKernel(reinterpret_cast<void*>(&icedem3d_kernel), dim3(grid),
                                                     dim3(kBlock), args, 0, s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(h->status_host, h->dev.status, sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  const int f = *h->status_host;
  if (f & kStatusNonfinite)
    return tdem::fail(&h->err, TDEM_ERR_NONFINITE, "non-finite DEM3D state; reduce dt or contact stiffness");
  if (f & kStatusContacts)
    return tdem::fail(&h->err, TDEM_ERR_CAPACITY,
                      "a particle overlaps more than " + std::to_string(kContacts) + " others");
  if (f & kStatusHistory)
    return tdem::fail(&h->err, TDEM_ERR_CAPACITY,
                      "a particle's friction history exceeds " + std::to_string(kHistory) + " partners");
  if (f & kStatusEscaped)
    return tdem::fail(&h->err, TDEM_ERR_CAPACITY, "a particle left the 2^20-cell hash range");
  if (f & kStatusBarrier)
    return tdem::fail(&h->err, TDEM_ERR_CUDA, "a grid barrier of the cooperative launch timed out");
  return TDEM_OK;
}

}  // namespace

extern "C" {

int tdem_icedem3d_max_particles(void) { return kMaxParticles; }

int tdem_icedem3d_create(const tdem_icedem3d_config* cfg, const tdem_icedem3d_topology* topo,
                         tdem_icedem3d** out) {
  if (!out) return TDEM_ERR_BADARG;
  *out = nullptr;
  if (!cfg || !topo) return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "null config or topology");
  const int n = cfg->n, nb = cfg->nbond;
  if (n < 2 || n > kMaxParticles)
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "n must be in 2.." + std::to_string(kMaxParticles));
  if (nb < 0) return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "nbond must be >= 0");
  if (cfg->n_branches < 0 || cfg->n_branches > TDEM_ICE3D_MAX_BRANCHES)
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "n_branches must be in 0..4");
  if (!(cfg->dt > 0.0) || !(cfg->mass > 0.0) || !(cfg->radius > 0.0))
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "dt, mass and radius must be positive");
  if (nb > 0 && (!topo->bond_i || !topo->bond_j || !topo->rest_length || !topo->reference ||
                 !topo->initial_normal))
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "bond topology arrays missing");
  if (!topo->pinv || !topo->full_rank)
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "per-particle pseudo-inverses missing");
  if (cfg->creep && !topo->creep_reference)
    return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "creep needs the per-bond reference force");
  // per-particle incidence: i side (ascending j), then j side (ascending i)
  std::vector<int> cnt_i(n, 0), cnt_j(n, 0);
  long long prev = -1;
  for (int b = 0; b < nb; ++b) {
    const int i = topo->bond_i[b], j = topo->bond_j[b];
    if (i < 0 || j <= i || j >= n)
      return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "bond " + std::to_string(b) + " is not 0 <= i < j < n");
    const long long key = (long long)i * n + j;
    if (key <= prev) return tdem::fail(&g_create_error3, TDEM_ERR_BADARG, "bonds must be sorted by i * n + j");
    prev = key;
    ++cnt_i[i];
    ++cnt_j[j];
  }
  std::vector<int> off(n + 1, 0), split(n);
  std::vector<int2> inc(2 * (size_t)nb);
  for (int k = 0; k < n; ++k) {
    off[k + 1] = off[k] + cnt_i[k] + cnt_j[k];
    split[k] = cnt_i[k];
  }
  std::vector<int> fi(n), fj(n);
  for (int k = 0; k < n; ++k) {
    fi[k] = off[k];
    fj[k] = off[k] + cnt_i[k];
  }
  for (int b = 0; b < nb; ++b) {
    const int i = topo->bond_i[b], j = topo->bond_j[b];
    inc[fi[i]++] = make_int2(b, j);
    inc[fj[j]++] = make_int2(b, i);
  }
  tdem_icedem3d* h = new tdem_icedem3d();
  h->cfg = *cfg;
  h->n = n;
  h->nb = nb;
  Dev& D = h->dev;
  unsigned H = 64;
  while (H < 2u * (unsigned)n) H <<= 1;
  D.barrier_spins = kBarrierSpins;
  D.hmask = H - 1;
  int rc = 0;
  auto fail_out = [&](int code) {
    g_create_error3 = h->err;
    destroy(h);
    return code;
  };
  if ((rc = dupload(h, &D.bi, topo->bond_i, nb)) || (rc = dupload(h, &D.bj, topo->bond_j, nb)) ||
      (rc = dupload(h, &D.rest, topo->rest_length, nb)) || (rc = dupload(h, &D.ref, topo->reference, 3 * (size_t)nb)) ||
      (rc = dupload(h, &D.inorm, topo->initial_normal, 3 * (size_t)nb)) ||
      (rc = dupload(h, &D.pinv, topo->pinv, 9 * (size_t)n)) ||
      (rc = dupload(h, &D.frank, topo->full_rank, (size_t)n)))
    return fail_out(rc);
  D.thr = nullptr;
  D.cref = nullptr;
  if (topo->threshold && (rc = dupload(h, &D.thr, topo->threshold, nb))) return fail_out(rc);
  if (topo->creep_reference && (rc = dupload(h, &D.cref, topo->creep_reference, nb))) return fail_out(rc);
  const int* p_off = nullptr;
  const int* p_split = nullptr;
  const int2* p_inc = nullptr;
  if ((rc = dupload(h, &p_off, off.data(), off.size())) || (rc = dupload(h, &p_split, split.data(), split.size())) ||
      (rc = dupload(h, &p_inc, inc.data(), inc.size())))
    return fail_out(rc);
  D.inc_off = p_off;
  D.inc_split = p_split;
  D.inc = p_inc;
  if ((rc = dalloc(h, &D.shear, n)) || (rc = dalloc(h, &D.abf, 3 * (size_t)nb)) || (rc = dalloc(h, &D.pkey, n)) ||
      (rc = dalloc(h, &D.pslot, n)) || (rc = dalloc(h, &D.hkey, 2 * (size_t)H)) ||
      (rc = dalloc(h, &D.hcnt, 2 * (size_t)H)) || (rc = dalloc(h, &D.hstart, H)) ||
      (rc = dalloc(h, &D.hfill, 2 * (size_t)H)) || (rc = dalloc(h, &D.members, n)) || (rc = dalloc(h, &D.ci_cnt, n)) ||
      (rc = dalloc(h, &D.ci_j, (size_t)n * kContacts)) || (rc = dalloc(h, &D.ci_v, (size_t)n * kContacts * 9)) ||
      (rc = dalloc(h, &D.ib_cnt, n)) || (rc = dalloc(h, &D.ib_key, (size_t)n * kContacts)) ||
      (rc = dalloc(h, &D.ib_idx, (size_t)n * kContacts)) || (rc = dalloc(h, &D.hist_old, n)) ||
      (rc = dalloc(h, &D.cellmin, n)) ||
      (rc = dalloc(h, &D.hist_cnt, n)) || (rc = dalloc(h, &D.hist_j, (size_t)n * kHistory)) ||
      (rc = dalloc(h, &D.hist_d, (size_t)n * kHistory * 3)) || (rc = dalloc(h, &D.ledger, TDEM_L3_COUNT)) ||
      (rc = dalloc(h, &D.status, 1)))
    return fail_out(rc);
  // cooperative grid: every block must be resident at once
  int dev = 0, sms = 0, coop = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, icedem3d_kernel, kBlock, 0) != cudaSuccess) {
    h->err = "device query failed";
    return fail_out(TDEM_ERR_CUDA);
  }
  if (!coop || per_sm < 1) {
    h->err = "the device does not support cooperative launches of the 3-D step kernel";
    return fail_out(TDEM_ERR_CUDA);
  }
  h->max_grid = sms * per_sm;
  if ((rc = dalloc(h, &D.bar_count, 1)) || (rc = dalloc(h, &D.bar_gen, 1)) || (rc = dalloc(h, &D.cursor, 2)) ||
      (rc = dalloc(h, &D.gflags, 2)) || (rc = dalloc(h, &D.part, (size_t)h->max_grid * kPartials)) ||
      (rc = dalloc(h, &D.pmin, 2 * (size_t)h->max_grid)) || (rc = dalloc(h, &D.pdiss, (size_t)h->max_grid)))
    return fail_out(rc);
  std::vector<double> led(TDEM_L3_COUNT, 0.0);
  led[TDEM_L3_MIN_BREAK_MARGIN] = 1e300;
  if (cudaMemcpy(D.ledger, led.data(), led.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(D.hist_cnt, 0, (size_t)n * sizeof(int)) != cudaSuccess ||
      cudaMemset(D.ci_cnt, 0, (size_t)n * sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&h->ledger_host, TDEM_L3_COUNT * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&h->status_host, sizeof(int)) != cudaSuccess) {
    h->err = "device initialisation failed";
    return fail_out(TDEM_ERR_CUDA);
  }
  *out = h;
  return TDEM_OK;
}

void tdem_icedem3d_destroy(tdem_icedem3d* h) { destroy(h); }

int tdem_icedem3d_forces(tdem_icedem3d* h, const tdem_icedem3d_state* st, const double* loads, double time,
                         int update_fracture, int update_history, double* out_force, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  if (!out_force) return tdem::fail(&h->err, TDEM_ERR_BADARG, "out_force is required");
  Out o{out_force, 1, update_fracture ? 1 : 0, update_history ? 1 : 0, 1, time, h->mapping};
  return launch(h, st, loads, o, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_icedem3d_step(tdem_icedem3d* h, const tdem_icedem3d_state* st, const double* loads, int64_t n_steps,
                       double time, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  if (n_steps < 1) return tdem::fail(&h->err, TDEM_ERR_BADARG, "n_steps must be >= 1");
  Out o{nullptr, 0, 1, 1, (long long)n_steps, time, h->mapping};
  return launch(h, st, loads, o, reinterpret_cast<cudaStream_t>(stream));
}

int tdem_icedem3d_set_barrier_spins(tdem_icedem3d* h, uint64_t spins) {
  if (!h) return TDEM_ERR_BADARG;
  h->dev.barrier_spins = (unsigned long long)spins;
  return TDEM_OK;
}

int tdem_icedem3d_set_mapping(tdem_icedem3d* h, int mapping) {
  if (!h) return TDEM_ERR_BADARG;
  if (mapping < TDEM_ICE3D_MAP_AUTO || mapping > TDEM_ICE3D_MAP_PARTICLE)
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "mapping must be TDEM_ICE3D_MAP_AUTO, _LANES or _PARTICLE");
  h->mapping = mapping;
  return TDEM_OK;
}

int tdem_icedem3d_read_ledger(tdem_icedem3d* h, double* out, int count, void* stream) {
  if (!h || !out || count < 0 || count > TDEM_L3_COUNT) return TDEM_ERR_BADARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(h->ledger_host, h->dev.ledger, TDEM_L3_COUNT * sizeof(double),
                                         cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  h->ledger_host[TDEM_L3_STATUS] = (double)*h->status_host;
  std::memcpy(out, h->ledger_host, count * sizeof(double));
  return TDEM_OK;
}

int tdem_icedem3d_read_contacts(tdem_icedem3d* h, int32_t* pairs, int64_t capacity, int64_t* count, void* stream) {
  if (!h || !count || capacity < 0 || (capacity > 0 && !pairs)) return TDEM_ERR_BADARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  std::vector<int> cnt(h->n), js((size_t)h->n * kContacts);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(cnt.data(), h->dev.ci_cnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(js.data(), h->dev.ci_j, js.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  int64_t m = 0;
  for (int k = 0; k < h->n; ++k)
    for (int c = 0; c < cnt[k]; ++c) {
      if (m < capacity) {
        pairs[2 * m] = k;
        pairs[2 * m + 1] = js[(size_t)k * kContacts + c];
      }
      ++m;
    }
  *count = m;
  if (m > capacity) return tdem::fail(&h->err, TDEM_ERR_CAPACITY, "contact buffer too small");
  return TDEM_OK;
}

int tdem_icedem3d_set_history(tdem_icedem3d* h, const int32_t* pairs, const double* disp, int64_t count,
                              void* stream) {
  if (!h || count < 0 || (count > 0 && (!pairs || !disp))) return TDEM_ERR_BADARG;
  const int n = h->n;
  std::vector<int> cnt(n, 0), js((size_t)n * kHistory, 0);
  std::vector<double> ds((size_t)n * kHistory * 3, 0.0);
  for (int64_t e = 0; e < count; ++e) {
    const int i = pairs[2 * e], j = pairs[2 * e + 1];
    if (i < 0 || j <= i || j >= n)
      return tdem::fail(&h->err, TDEM_ERR_BADARG, "history pair " + std::to_string(e) + " is not 0 <= i < j < n");
    if (cnt[i] == kHistory)
      return tdem::fail(&h->err, TDEM_ERR_CAPACITY,
                        "particle " + std::to_string(i) + " has more than " + std::to_string(kHistory) + " partners");
    for (int q = 0; q < cnt[i]; ++q)
      if (js[(size_t)i * kHistory + q] == j)
        return tdem::fail(&h->err, TDEM_ERR_BADARG, "duplicate history pair");
    const size_t slot = (size_t)i * kHistory + cnt[i]++;
    js[slot] = j;
    for (int c = 0; c < 3; ++c) ds[3 * slot + c] = disp[3 * e + c];
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpy(h->dev.hist_cnt, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice));
  TDEM_CUDA_TRY(&h->err, cudaMemcpy(h->dev.hist_j, js.data(), js.size() * sizeof(int), cudaMemcpyHostToDevice));
  TDEM_CUDA_TRY(&h->err, cudaMemcpy(h->dev.hist_d, ds.data(), ds.size() * sizeof(double), cudaMemcpyHostToDevice));
  return TDEM_OK;
}

int tdem_icedem3d_read_history(tdem_icedem3d* h, int32_t* pairs, double* disp, int64_t capacity, int64_t* count,
                               void* stream) {
  if (!h || !count || capacity < 0 || (capacity > 0 && (!pairs || !disp))) return TDEM_ERR_BADARG;
  const int n = h->n;
  std::vector<int> cnt(n), js((size_t)n * kHistory);
  std::vector<double> ds((size_t)n * kHistory * 3);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(cnt.data(), h->dev.hist_cnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(js.data(), h->dev.hist_j, js.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(ds.data(), h->dev.hist_d, ds.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  int64_t m = 0;
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < cnt[i]; ++q) {
      const size_t slot = (size_t)i * kHistory + q;
      if (m < capacity) {
        pairs[2 * m] = i;
        pairs[2 * m + 1] = js[slot];
        for (int c = 0; c < 3; ++c) disp[3 * m + c] = ds[3 * slot + c];
      }
      ++m;
    }
  *count = m;
  if (m > capacity) return tdem::fail(&h->err, TDEM_ERR_CAPACITY, "history buffer too small");
  return TDEM_OK;
}

// ---------------------------------------------------------------------------
// The universal restitution curve of a Hertz spring with the Tsuji dashpot and
// its inverse (contact_calibration.py:60-248): the similarity ODE
// u'' = -max(u^(3/2) + 2 zeta u^(1/4) u', 0), u(0) = 0, u'(0) = sqrt(4/5), is
// integrated by classical RK4 at dimensionless step 1e-4 (at most 50 time
// units); the exit rate comes from the cubic Hermite interpolant of the last
// step, located by bisection; the requested restitution is inverted by a
// secant iteration from the linear spring-dashpot mapping. Host arithmetic in
// the reference's operation order, so the damping ratio has its bits.
// ---------------------------------------------------------------------------
namespace {

double hertz_accel(double u, double w, double zeta) {
  if (u <= 0.0) return 0.0;
  const double f = u * std::sqrt(u) + ((2.0 * zeta) * std::pow(u, 0.25)) * w;
  return f > 0.0 ? -f : 0.0;
}

double hermite_exit_rate(double u0, double w0, double u1, double w1, double dt) {
  auto u_of = [&](double th) {
    const double t2 = th * th, t3 = t2 * th;
    return (((2.0 * t3 - 3.0 * t2 + 1.0) * u0 + ((t3 - 2.0 * t2 + th) * dt) * w0) + (-2.0 * t3 + 3.0 * t2) * u1) +
           ((t3 - t2) * dt) * w1;
  };
  auto du_of = [&](double th) {
    const double t2 = th * th;
    return (((6.0 * t2 - 6.0 * th) * u0 + ((3.0 * t2 - 4.0 * th + 1.0) * dt) * w0) + (-6.0 * t2 + 6.0 * th) * u1) +
           ((3.0 * t2 - 2.0 * th) * dt) * w1;
  };
  double lo = 0.0, hi = 1.0;
  for (int it = 0; it < 60; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (u_of(mid) > 0.0) lo = mid;
    else hi = mid;
    if (hi - lo < 1e-14) break;
  }
  return du_of(0.5 * (lo + hi)) / dt;
}

double hertz_restitution(double zeta) {
  if (zeta == 0.0) return 1.0;
  const double dt = 1.0e-4;
  const double w0 = std::sqrt(4.0 / 5.0);
  double u = 0.0, w = w0;
  bool seen = false;
  const long n_max = (long)(50.0 / dt) + 1;
  for (long it = 0; it < n_max; ++it) {
    const double k1u = w, k1w = hertz_accel(u, w, zeta);
    const double u2 = u + (0.5 * dt) * k1u, w2 = w + (0.5 * dt) * k1w;
    const double k2u = w2, k2w = hertz_accel(u2, w2, zeta);
    const double u3 = u + (0.5 * dt) * k2u, w3 = w + (0.5 * dt) * k2w;
    const double k3u = w3, k3w = hertz_accel(u3, w3, zeta);
    const double u4 = u + dt * k3u, w4 = w + dt * k3w;
    const double k4u = w4, k4w = hertz_accel(u4, w4, zeta);
    const double un = u + (dt * (((k1u + 2.0 * k2u) + 2.0 * k3u) + k4u)) / 6.0;
    const double wn = w + (dt * (((k1w + 2.0 * k2w) + 2.0 * k3w) + k4w)) / 6.0;
    if (u > 0.0) seen = true;
    if (seen && un <= 0.0 && wn < 0.0)
      return std::min(1.0, std::max(0.0, std::fabs(hermite_exit_rate(u, w, un, wn, dt)) / w0));
    u = un;
    w = wn;
  }
  return 0.0;
}

}  // namespace

int tdem_hertz_damping_ratio(double restitution, double* zeta_out) {
  if (!zeta_out || !(restitution > 0.0 && restitution <= 1.0)) return TDEM_ERR_BADARG;
  if (restitution == 1.0) {
    *zeta_out = 0.0;
    return TDEM_OK;
  }
  const double pi = 3.141592653589793;
  const double a = -std::log(restitution);
  double z0 = a / std::sqrt(std::pow(pi, 2.0) + std::pow(a, 2.0));
  double f0 = hertz_restitution(z0) - restitution;
  double z1 = f0 > 0.0 ? z0 * 1.118 : z0 * (1.0 - 0.05);
  double f1 = hertz_restitution(z1) - restitution;
  for (int it = 0; it < 80; ++it) {
    if (std::fabs(f1) <= 1.0e-10) break;
    const double denom = f1 - f0;
    if (denom == 0.0) break;
    double z2 = z1 - (f1 * (z1 - z0)) / denom;
    if (!(0.0 < z2 && z2 < 1.0)) z2 = z0 < z1 ? 0.5 * (z0 + z1) : 0.5 * (z1 + z0);
    const double f2 = hertz_restitution(z2) - restitution;
    z0 = z1;
    f0 = f1;
    z1 = z2;
    f1 = f2;
  }
  *zeta_out = z1;
  return TDEM_OK;
}

int tdem_icedem3d_last_error(const tdem_icedem3d* h, char* buf, size_t len) {
  if (!buf || len == 0) return TDEM_ERR_BADARG;
  const std::string& e = h ? h->err : g_create_error3;
  const size_t m = std::min(len - 1, e.size());
  std::memcpy(buf, e.data(), m);
  buf[m] = '\0';
  return TDEM_OK;
}

}  // extern "C"
