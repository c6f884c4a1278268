// Reference-mode engine: the FP64 2-D bonded-disc step of the reference's
// IceDEM (src/tensordem/dem.py), on sm_103a.
//
// Design. One CTA owns one instance and runs many steps per launch; the
// instance's positions, velocities, per-disc shear strain and forces sit in
// shared memory between the phases of a step, so a step costs no global
// round trip beyond the caller-owned state writes. Each disc's force is
// accumulated by one thread in exactly the order of the reference's two
// index_add_ calls (dem.py:290-292): partners j > k ascending (disc k is the
// pair's i), then partners i < k ascending (disc k is the pair's j). Pairs
// that are neither alive bonds nor overlapping contribute +-0 in the
// reference and are skipped here after an FP32 distance prefilter. All block
// reductions run in a fixed order, so reruns are bitwise identical.
//
// This translation unit is compiled with --fmad=false: the reference runs
// one torch op per arithmetic step, each rounded separately. The one fused
// operation is torch's CPU vector_norm, which sums the squares of a 2-vector
// as fma(y, y, x*x); distances are computed that way, with fma() explicitly.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"

namespace tdem {
namespace icedem {

constexpr int kMaxDiscs = 2048;
constexpr int kMaxHull = 64;

struct Params {
  int n;
  int nbond;
  int hull_m;  // 0: circular tool
  double radius, mass, kb, kc, eps_t, eps_s, cdamp, drag, tool_radius, dt;
  double tool_start_x, tool_start_y, tool_vel_x, tool_vel_y;
  double hull_start_x, hull_start_y, hull_vel_x, hull_vel_y;
};

// Row-major 2x2 matrix.
struct Mat2 {
  double x, y, z, w;
};

struct Topo {
  const int* bi;          // (B) bond endpoint i (< j)
  const int* bj;          // (B)
  const long long* bpair; // (B) pair index of the bond
  const double* rest;     // (B) rest length = initial distance
  const double2* ref;     // (B) reference bond vector x0[j] - x0[i]
  const int* inc_off;     // (n+1) per-disc incidence offsets
  const int* inc_bond;    // (2B) bond ids in reference accumulation order
  const int* inc_other;   // (2B) partner disc of that bond
  const Mat2* pinv;       // (n) pseudo-inverse of the bond covariance (row major)
  const double2* hull;    // (hull_m) local hull vertices
  const double* kcoef;    // (B) per-bond stiffness (N/m), or null: the config's stiffness for every bond
};

struct Mailbox {
  int status;      // TDEM_OK or TDEM_ERR_NONFINITE
  int steps_done;  // steps completed by the last launch
};

// ---------------------------------------------------------------------------
// Tool / hull contact for one disc. Returns the disc force and adds the
// disc's share of the tool dissipation (dem.py:294-339, hull_contact.py:7-75).
// ---------------------------------------------------------------------------
__device__ inline double2 tool_contact(const Params& P, const Topo& T, double2 p, double2 v,
                                       double time, double& tool_diss) {
  const double eps = 2.220446049250313e-16;
  double2 normal, tv;
  double overlap;
  if (P.hull_m == 0) {
    const double tx = P.tool_start_x + time * P.tool_vel_x;
    const double ty = P.tool_start_y + time * P.tool_vel_y;
    const double dx = p.x - tx, dy = p.y - ty;
    const double dist = sqrt(fma(dy, dy, dx * dx));
    const double dcl = fmax(dist, eps);
    if (dist > 0.0) {
      normal = make_double2(dx / dcl, dy / dcl);
    } else {
      normal = make_double2(0.0, -1.0);
    }
    overlap = fmax(P.radius + P.tool_radius - dist, 0.0);
    tv = make_double2(P.tool_vel_x, P.tool_vel_y);
  } else {
    const double ox = P.hull_start_x + time * P.hull_vel_x;
    const double oy = P.hull_start_y + time * P.hull_vel_y;
    tv = make_double2(P.hull_vel_x, P.hull_vel_y);
    double best_d2 = 0.0, bdx = 0.0, bdy = 0.0, bsx = 0.0, bsy = 0.0, blen2 = 1.0;
    for (int m = 0; m + 1 < P.hull_m; ++m) {
      const double ax = T.hull[m].x + ox, ay = T.hull[m].y + oy;
      const double sx = (T.hull[m + 1].x + ox) - ax, sy = (T.hull[m + 1].y + oy) - ay;
      const double len2 = sx * sx + sy * sy;
      const double rx = p.x - ax, ry = p.y - ay;
      double frac = (rx * sx + ry * sy) / len2;
      frac = fmin(fmax(frac, 0.0), 1.0);
      const double cx = ax + frac * sx, cy = ay + frac * sy;
      const double dx = p.x - cx, dy = p.y - cy;
      const double d2 = dx * dx + dy * dy;
      if (m == 0 || d2 < best_d2) {  // first minimum wins, as argmin does
        best_d2 = d2;
        bdx = dx;
        bdy = dy;
        bsx = sx;
        bsy = sy;
        blen2 = len2;
      }
    }
    const double dist = sqrt(best_d2);
    const double sl = sqrt(blen2);
    double tx = bsx / sl, ty = bsy / sl;
    if (tx < 0.0 || (tx == 0.0 && ty < 0.0)) {
      tx = -tx;
      ty = -ty;
    }
    double fx = -ty, fy = tx;
    const double approach = (v.x - tv.x) * fx + (v.y - tv.y) * fy;
    if (approach > 0.0) {
      fx = -fx;
      fy = -fy;
    }
    if (dist > eps) {
      const double dcl = fmax(dist, eps);
      normal = make_double2(bdx / dcl, bdy / dcl);
    } else {
      normal = make_double2(fx, fy);
    }
    overlap = fmax(P.radius + P.tool_radius - dist, 0.0);
  }
  const double rvx = v.x - tv.x, rvy = v.y - tv.y;
  const double speed = rvx * normal.x + rvy * normal.y;
  double mag = fmax(P.kc * overlap - P.cdamp * speed, 0.0);
  if (!(overlap > 0.0)) mag = 0.0;
  const double2 f = make_double2(mag * normal.x, mag * normal.y);
  // conservative part: same geometry, zero damping (overlap is clamped >= 0)
  const double cmag = P.kc * overlap;
  const double cfx = cmag * normal.x;
  const double cfy = cmag * normal.y;
  tool_diss += (f.x - cfx) * rvx;
  tool_diss += (f.y - cfy) * rvy;
  return f;
}

// Distance from a disc centre to the tool at `time`: the circle's centre, or
// the nearest point of the hull polyline (the first nearest segment wins).
__device__ inline double tool_distance(const Params& P, const Topo& T, double2 p, double time) {
  if (P.hull_m == 0) {
    const double dx = p.x - (P.tool_start_x + time * P.tool_vel_x);
    const double dy = p.y - (P.tool_start_y + time * P.tool_vel_y);
    return sqrt(fma(dy, dy, dx * dx));
  }
  const double ox = P.hull_start_x + time * P.hull_vel_x;
  const double oy = P.hull_start_y + time * P.hull_vel_y;
  double best = 0.0;
  for (int m = 0; m + 1 < P.hull_m; ++m) {
    const double ax = T.hull[m].x + ox, ay = T.hull[m].y + oy;
    const double sx = (T.hull[m + 1].x + ox) - ax, sy = (T.hull[m + 1].y + oy) - ay;
    double frac = ((p.x - ax) * sx + (p.y - ay) * sy) / (sx * sx + sy * sy);
    frac = fmin(fmax(frac, 0.0), 1.0);
    const double dx = p.x - (ax + frac * sx), dy = p.y - (ay + frac * sy);
    const double d = sqrt(fma(dy, dy, dx * dx));
    if (m == 0 || d < best) best = d;
  }
  return best;
}

// Stored mechanical energy of a state (the reference's mechanical_energy,
// dem.py:603-624): kinetic, the springs of the intact bonds (per-bond
// stiffness when set), the penalty energy of every overlapping pair that is not
// an intact bond, and the tool's penalty energy. One CTA; every sum in a fixed
// order. out: kinetic, bond, pair contact, tool contact, total (J).
__global__ void __launch_bounds__(512) icedem_energy_kernel(Params P, Topo T, const double2* __restrict__ pos,
                                                            const double2* __restrict__ vel,
                                                            const bool* __restrict__ alive, double time,
                                                            double* __restrict__ out) {
  __shared__ double red[4 * 16];
  const int n = P.n, tid = threadIdx.x, nt = blockDim.x;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};  // sum |v|^2, bond, sum overlap^2 (pairs), (tool)
  for (int k = tid; k < n; k += nt) {
    const double2 v = vel[k];
    acc[0] += v.x * v.x + v.y * v.y;
    const double ov = fmax(P.radius + P.tool_radius - tool_distance(P, T, pos[k], time), 0.0);
    acc[3] += ov * ov;
  }
  for (int b = tid; b < P.nbond; b += nt) {
    if (!alive[T.bpair[b]]) continue;
    const double2 a = pos[T.bi[b]], c = pos[T.bj[b]];
    const double dx = c.x - a.x, dy = c.y - a.y;
    const double ext = sqrt(fma(dy, dy, dx * dx)) - T.rest[b];
    acc[1] += 0.5 * (T.kcoef ? T.kcoef[b] : P.kb) * (ext * ext);
  }
  // every pair (i < j) closer than two radii that is not an intact bond; the
  // row of disc i starts at pair index i n - i (i + 1) / 2
  const double reach = 2.0 * P.radius;
  for (int i = tid; i < n; i += nt) {
    const double2 a = pos[i];
    const long long row = (long long)i * n - (long long)i * (i + 1) / 2 - (i + 1);
    for (int j = i + 1; j < n; ++j) {
      const double2 c = pos[j];
      const double dx = c.x - a.x, dy = c.y - a.y;
      if (fabs(dx) >= reach || fabs(dy) >= reach) continue;
      const double ov = fmax(reach - sqrt(fma(dy, dy, dx * dx)), 0.0);
      if (ov > 0.0 && !alive[row + j]) acc[2] += ov * ov;
    }
  }
  double tot[4];
  block_sum_f64<4>(acc, red, tot);
  if (tid == 0) {
    const double kinetic = 0.5 * P.mass * tot[0];
    const double pair = 0.5 * P.kc * tot[2];
    const double tool = 0.5 * P.kc * tot[3];
    out[0] = kinetic;
    out[1] = tot[1];
    out[2] = pair;
    out[3] = tool;
    out[4] = kinetic + tot[1] + pair + tool;
  }
}

// Fragments: connected components of the intact bonds (isolated discs are
// components of their own), each disc labelled with the smallest disc id of
// its component. One CTA, parents in shared memory: every intact bond hooks
// the larger of its two roots under the smaller (atomicMin keeps parents
// decreasing, so a root is always its component's smallest id), then every
// parent pointer is jumped to its root; rounds repeat until no bond joins two
// roots. A component of n discs needs at most n rounds; `*rounds_out` gets the
// count, or -1 if the bound was reached.
__global__ void __launch_bounds__(512) icedem_fragment_kernel(Params P, Topo T, const bool* __restrict__ alive,
                                                              int* __restrict__ label, int* __restrict__ rounds_out) {
  extern __shared__ int par[];
  const int n = P.n, tid = threadIdx.x, nt = blockDim.x;
  for (int k = tid; k < n; k += nt) par[k] = k;
  __syncthreads();
  int rounds = 0;
  bool joined = true;
  while (joined && rounds <= n) {
    bool any = false;
    for (int b = tid; b < P.nbond; b += nt) {
      if (!alive[T.bpair[b]]) continue;
      int ra = T.bi[b], rb = T.bj[b];
      while (par[ra] != ra) ra = par[ra];
      while (par[rb] != rb) rb = par[rb];
      if (ra != rb) {
        atomicMin(&par[max(ra, rb)], min(ra, rb));
        any = true;
      }
    }
    __syncthreads();
    for (int k = tid; k < n; k += nt) {
      int r = par[k];
      while (par[r] != r) r = par[r];
      par[k] = r;
    }
    joined = __syncthreads_or(any) != 0;
    ++rounds;
  }
  for (int k = tid; k < n; k += nt) label[k] = par[k];
  if (tid == 0) *rounds_out = joined ? -1 : rounds;
}

// ---------------------------------------------------------------------------
// The fused step kernel. mode 0: n_steps full steps; mode 1: one force
// evaluation (dem.py:226-345) written to out_force / out_reaction.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512) icedem_kernel(Params P, Topo T, tdem_icedem_state S,
                                                      const double2* __restrict__ loads, int mode,
                                                      int n_steps, double time,
                                                      double2* __restrict__ out_force,
                                                      double* __restrict__ out_reaction,
                                                      double* __restrict__ ledger,
                                                      Mailbox* __restrict__ mbox) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = P.n;
  double2* spos = reinterpret_cast<double2*>(smem_raw);
  double2* svel = spos + n;
  double2* sforce = svel + n;
  double* sshear = reinterpret_cast<double*>(sforce + n);
  float2* sposf = reinterpret_cast<float2*>(sshear + n);
  double* red = reinterpret_cast<double*>(sposf + n + (n & 1));  // reductions

  double2* gpos = reinterpret_cast<double2*>(S.positions);
  double2* gvel = reinterpret_cast<double2*>(S.velocities);
  const double2* gpos0 = reinterpret_cast<const double2*>(S.initial_positions);
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ int s_bad;
  if (tid == 0) s_bad = 0;

  for (int k = tid; k < n; k += nt) {
    const double2 p = gpos[k];
    spos[k] = p;
    svel[k] = gvel[k];
    sposf[k] = make_float2((float)p.x, (float)p.y);
  }
  __syncthreads();

  const double two_r = 2.0 * P.radius;
  // Prefilter for pairs that are not alive bonds: only a pair closer than 2r
  // can carry a force. FP32 squared distances are accurate to ~1e-7 relative,
  // far inside the 1e-3 guard band.
  const float pre2 = (float)(two_r * two_r) * 1.001f + 1e-30f;
  const double eps = 2.220446049250313e-16;
  double min_margin = 1e300;
  int steps_done = 0;
  const int total = (mode == 1) ? 1 : n_steps;

  for (int step = 0; step < total; ++step) {
    // ---- phase 1: objective local shear strain per disc (dem.py:182-208)
    for (int k = tid; k < n; k += nt) {
      double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
      for (int e = T.inc_off[k]; e < T.inc_off[k + 1]; ++e) {
        const int b = T.inc_bond[e];
        const int i = T.bi[b], j = T.bj[b];
        const double2 r = T.ref[b];
        const double cx = spos[j].x - spos[i].x;
        const double cy = spos[j].y - spos[i].y;
        c00 += cx * r.x;
        c01 += cx * r.y;
        c10 += cy * r.x;
        c11 += cy * r.y;
      }
      const Mat2 q = T.pinv[k];
      const double f00 = c00 * q.x + c01 * q.z;
      const double f01 = c00 * q.y + c01 * q.w;
      const double f10 = c10 * q.x + c11 * q.z;
      const double f11 = c10 * q.y + c11 * q.w;
      const double e00 = 0.5 * ((f00 * f00 + f10 * f10) - 1.0);
      const double e01 = 0.5 * (f00 * f01 + f10 * f11);
      const double e11 = 0.5 * ((f01 * f01 + f11 * f11) - 1.0);
      const double dd = e00 - e11;
      sshear[k] = sqrt(dd * dd + 4.0 * (e01 * e01));
    }
    __syncthreads();

    // ---- phase 2: break test and irreversible commit (dem.py:243-277)
    double brk[3] = {0.0, 0.0, 0.0};  // released, acquired, per-bond stiffness correction
    int any_break = 0;
    for (int b = tid; b < P.nbond; b += nt) {
      const long long p = T.bpair[b];
      if (!S.alive[p]) continue;
      const int i = T.bi[b], j = T.bj[b];
      const double dx = spos[j].x - spos[i].x, dy = spos[j].y - spos[i].y;
      const double d = sqrt(fma(dy, dy, dx * dx));
      const double ext = d - T.rest[b];
      const double ts = ext / T.rest[b];
      const double bs = 0.5 * (sshear[i] + sshear[j]);
      const bool tf = ts > P.eps_t;
      const bool sf = bs > P.eps_s;
      if (tf || sf) {
        S.alive[p] = 0;
        S.failure_mode[p] = (uint8_t)((tf ? 1 : 0) + 2 * (sf ? 1 : 0));
        S.failure_time_s[p] = time;
        S.failure_extension_m[p] = ext;
        const double energy = (0.5 * P.kb) * (ext * ext);
        S.failure_energy_J[p] = energy;
        if (T.kcoef) {
          // per-bond stiffness: the released energy of the actual spring law
          // (calibrated_dem.py:80-84), booked after the base energy
          const double corr = (0.5 * (T.kcoef[b] - P.kb)) * (ext * ext);
          S.failure_energy_J[p] = energy + corr;
          brk[2] += corr;
        }
        const double ov = fmax(two_r - d, 0.0);
        brk[0] += energy;
        brk[1] += (0.5 * P.kc) * (ov * ov);
        any_break = 1;
      } else {
        min_margin = fmin(min_margin, fmin((P.eps_t - ts) / P.eps_t, (P.eps_s - bs) / P.eps_s));
      }
    }
    if (__syncthreads_or(any_break)) {
      double tot[3];
      block_sum_f64<3>(brk, red, tot);
      if (tid == 0) {
        ledger[TDEM_L_FRACTURE_RELEASE] += tot[0];
        ledger[TDEM_L_CONTACT_ACQUIRED] += tot[1];
        if (T.kcoef) ledger[TDEM_L_FRACTURE_RELEASE] += tot[2];
      }
    }
    __syncthreads();

    // ---- phase 3: pair, drag, tool and load forces (dem.py:278-345)
    // partial sums: tool force (2), support (2), sum v (2), loads (2),
    // pair dissipation, tool dissipation, sum v^2, load moment
    double acc[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) acc[q] = 0.0;
    for (int k = tid; k < n; k += nt) {
      const double2 pk = spos[k];
      const double2 vk = svel[k];
      const float2 pkf = sposf[k];
      double fx = (-P.drag) * vk.x;
      double fy = (-P.drag) * vk.y;
      int cur = T.inc_off[k];
      const int cur_end = T.inc_off[k + 1];
      for (int t = 1; t < n; ++t) {
        int j = k + t;
        if (j >= n) j -= n;  // k+1..n-1, then 0..k-1
        bool alive = false;
        if (cur < cur_end && T.inc_other[cur] == j) {
          alive = S.alive[T.bpair[T.inc_bond[cur]]] != 0;
          ++cur;
        }
        if (!alive) {
          const float ddx = sposf[j].x - pkf.x, ddy = sposf[j].y - pkf.y;
          if (ddx * ddx + ddy * ddy > pre2) continue;
        }
        const int lo = k < j ? k : j;
        const int hi = k < j ? j : k;
        const double dx = spos[hi].x - spos[lo].x;
        const double dy = spos[hi].y - spos[lo].y;
        const double d = sqrt(fma(dy, dy, dx * dx));
        double nx, ny;
        if (d > 0.0) {
          const double dcl = fmax(d, eps);
          nx = dx / dcl;
          ny = dy / dcl;
        } else {
          const double ix = gpos0[hi].x - gpos0[lo].x, iy = gpos0[hi].y - gpos0[lo].y;
          const double id = sqrt(fma(iy, iy, ix * ix));
          nx = ix / id;
          ny = iy / id;
        }
        double mag;
        if (alive) {
          // alive bonds exist only between bonded pairs: the rest length is the bond's
          mag = P.kb * (d - T.rest[T.inc_bond[cur - 1]]);
        } else {
          const double ov = fmax(two_r - d, 0.0);
          if (!(ov > 0.0)) continue;
          const double vn = (svel[hi].x - svel[lo].x) * nx + (svel[hi].y - svel[lo].y) * ny;
          const double rep = fmax(P.kc * ov - P.cdamp * vn, 0.0);
          mag = -rep;
          if (k == lo) acc[8] += (rep - P.kc * ov) * (-vn);
        }
        const double pfx = mag * nx, pfy = mag * ny;
        if (k == lo) {
          fx += pfx;
          fy += pfy;
        } else {
          fx += -pfx;
          fy += -pfy;
        }
      }
      double tdiss = 0.0;
      const double2 tf = tool_contact(P, T, pk, vk, time, tdiss);
      acc[0] += tf.x;
      acc[1] += tf.y;
      acc[9] += tdiss;
      fx += tf.x;
      fy += tf.y;
      if (loads) {
        const double2 L = loads[k];
        fx += L.x;
        fy += L.y;
        acc[6] += L.x;
        acc[7] += L.y;
        acc[11] += pk.x * L.y - pk.y * L.x;
      }
      if (T.kcoef) {
        // per-bond stiffness (calibrated_dem.py:70-79): after the base force,
        // (k_b - k) * extension * n on each surviving bond, first the bonds
        // where this disc is i (ascending j), then those where it is j
        // (ascending i), which is the order of the incidence list
        for (int e = T.inc_off[k]; e < T.inc_off[k + 1]; ++e) {
          const int b = T.inc_bond[e];
          if (!S.alive[T.bpair[b]]) continue;
          const int j = T.inc_other[e];
          const int lo = k < j ? k : j;
          const int hi = k < j ? j : k;
          const double dx = spos[hi].x - spos[lo].x;
          const double dy = spos[hi].y - spos[lo].y;
          const double d = sqrt(fma(dy, dy, dx * dx));
          double nx, ny;
          if (d > 0.0) {
            const double dcl = fmax(d, eps);
            nx = dx / dcl;
            ny = dy / dcl;
          } else {
            const double ix = gpos0[hi].x - gpos0[lo].x, iy = gpos0[hi].y - gpos0[lo].y;
            const double id = sqrt(fma(iy, iy, ix * ix));
            nx = ix / id;
            ny = iy / id;
          }
          const double m = (T.kcoef[b] - P.kb) * (d - T.rest[b]);
          if (k == lo) {
            fx += m * nx;
            fy += m * ny;
          } else {
            fx += -(m * nx);
            fy += -(m * ny);
          }
        }
      }
      sforce[k] = make_double2(fx, fy);
      if (S.fixed[k]) {
        acc[2] += fx;
        acc[3] += fy;
      }
      acc[4] += vk.x;
      acc[5] += vk.y;
      acc[10] += vk.x * vk.x;
      acc[10] += vk.y * vk.y;
    }
    double tot[12];
    block_sum_f64<12>(acc, red, tot);
    // tot valid in thread 0
    double rx = 0.0, ry = 0.0;
    if (tid == 0) {
      rx = -tot[0];
      ry = -tot[1];
      const double tvx = P.hull_m ? P.hull_vel_x : P.tool_vel_x;
      const double tvy = P.hull_m ? P.hull_vel_y : P.tool_vel_y;
      const double damping_power = (tot[8] + (-tot[9])) + P.drag * tot[10];
      const double tool_power = -(rx * tvx + ry * tvy);
      ledger[TDEM_L_DAMPING_POWER] = damping_power;
      ledger[TDEM_L_TOOL_POWER] = tool_power;
      if (mode == 1) {
        out_reaction[0] = rx;
        out_reaction[1] = ry;
      }
    }
    if (mode == 1) {
      for (int k = tid; k < n; k += nt) out_force[k] = sforce[k];
      steps_done = 0;
      break;
    }

    // ---- phase 4: semi-implicit Euler and the ledger (dem.py:347-382)
    double wsum[2] = {0.0, 0.0};  // external work, non-finite flag
    for (int k = tid; k < n; k += nt) {
      const double2 F = sforce[k];
      const double2 v0 = svel[k];
      const double2 p0 = spos[k];
      double vx = v0.x + (P.dt * F.x) / P.mass;
      double vy = v0.y + (P.dt * F.y) / P.mass;
      const bool fixed = S.fixed[k] != 0;
      if (fixed) {
        vx = 0.0;
        vy = 0.0;
      }
      double px = p0.x + P.dt * vx;
      double py = p0.y + P.dt * vy;
      if (fixed) {
        px = gpos0[k].x;
        py = gpos0[k].y;
      }
      if (loads) {
        const double2 L = loads[k];
        wsum[0] += L.x * (px - p0.x);
        wsum[0] += L.y * (py - p0.y);
      }
      if (!(isfinite(px) && isfinite(py) && isfinite(vx) && isfinite(vy))) wsum[1] = 1.0;
      spos[k] = make_double2(px, py);
      svel[k] = make_double2(vx, vy);
      sposf[k] = make_float2((float)px, (float)py);
      gpos[k] = spos[k];
      gvel[k] = svel[k];
    }
    double wt[2];
    block_sum_f64<2>(wsum, red, wt);
    if (tid == 0) {
      const double dt = P.dt;
      const double sup_x = -tot[2], sup_y = -tot[3];
      const double drag_x = (-P.drag) * tot[4], drag_y = (-P.drag) * tot[5];
      const double ext_x = tot[6], ext_y = tot[7];
      ledger[TDEM_L_EXTERNAL_IMPULSE_X] = ledger[TDEM_L_EXTERNAL_IMPULSE_X] + dt * ext_x;
      ledger[TDEM_L_EXTERNAL_IMPULSE_Y] = ledger[TDEM_L_EXTERNAL_IMPULSE_Y] + dt * ext_y;
      ledger[TDEM_L_SUPPORT_IMPULSE_X] = ledger[TDEM_L_SUPPORT_IMPULSE_X] + dt * sup_x;
      ledger[TDEM_L_SUPPORT_IMPULSE_Y] = ledger[TDEM_L_SUPPORT_IMPULSE_Y] + dt * sup_y;
      ledger[TDEM_L_DRAG_IMPULSE_X] = ledger[TDEM_L_DRAG_IMPULSE_X] + dt * drag_x;
      ledger[TDEM_L_DRAG_IMPULSE_Y] = ledger[TDEM_L_DRAG_IMPULSE_Y] + dt * drag_y;
      ledger[TDEM_L_TOOL_IMPULSE_X] = ledger[TDEM_L_TOOL_IMPULSE_X] + dt * (-rx);
      ledger[TDEM_L_TOOL_IMPULSE_Y] = ledger[TDEM_L_TOOL_IMPULSE_Y] + dt * (-ry);
      const double work = loads ? wt[0] : 0.0;
      ledger[TDEM_L_EXTERNAL_WORK] += work;
      ledger[TDEM_L_TOOL_WORK] += dt * ledger[TDEM_L_TOOL_POWER];
      ledger[TDEM_L_DAMPING_DISSIPATION] += dt * ledger[TDEM_L_DAMPING_POWER];
      ledger[TDEM_L_LAST_SUPPORT_X] = sup_x;
      ledger[TDEM_L_LAST_SUPPORT_Y] = sup_y;
      ledger[TDEM_L_LAST_REACTION_X] = rx;
      ledger[TDEM_L_LAST_REACTION_Y] = ry;
      ledger[TDEM_L_LAST_EXTERNAL_X] = ext_x;
      ledger[TDEM_L_LAST_EXTERNAL_Y] = ext_y;
      ledger[TDEM_L_LAST_EXTERNAL_WORK] = work;
      ledger[TDEM_L_LAST_EXTERNAL_MOMENT] = loads ? tot[11] : 0.0;
      ledger[TDEM_L_LAST_TIME_START] = time;
      ledger[TDEM_L_LAST_TIME_END] = time + dt;
    }
    time = time + P.dt;
    steps_done = step + 1;
    // broadcast the non-finite verdict of this step from thread 0 to the block
    if (tid == 0) s_bad = (wt[1] > 0.0) ? 1 : 0;
    __syncthreads();
    if (s_bad) break;
  }

  const double m = block_min_f64(min_margin, red);
  if (tid == 0) {
    ledger[TDEM_L_MIN_BREAK_MARGIN] = fmin(ledger[TDEM_L_MIN_BREAK_MARGIN], m);
    mbox->steps_done = steps_done;
    mbox->status = s_bad ? TDEM_ERR_NONFINITE : TDEM_OK;
  }
}

}  // namespace icedem
}  // namespace tdem

// ===========================================================================
// Host side: topology build and the C ABI
// ===========================================================================

struct tdem_icedem {
  tdem::icedem::Params P{};
  int n = 0, nbond = 0;
  long long npairs = 0;
  std::vector<long long> bpair_host;
  // device buffers
  int *bi = nullptr, *bj = nullptr, *inc_off = nullptr, *inc_bond = nullptr, *inc_other = nullptr;
  long long* bpair = nullptr;
  double* rest = nullptr;
  double2* ref = nullptr;
  tdem::icedem::Mat2* pinv = nullptr;
  double2* hull = nullptr;
  double* kcoef = nullptr;  // per-bond stiffness, null unless set
  double* ledger = nullptr;
  double* energy = nullptr;  // 5 doubles: the energy kernel's output
  void* scratch = nullptr;   // fragment labels (kMaxDiscs ints) and a round count
  tdem::icedem::Mailbox* mbox = nullptr;
  tdem::icedem::Mailbox* mbox_host = nullptr;
  double* ledger_host = nullptr;
  int threads = 32;
  size_t smem = 0;
  std::string err;
};

namespace {

std::string g_create_error;

// Moore-Penrose pseudo-inverse of the symmetric positive semi-definite matrix
// [[a, b], [b, c]] through its eigen-decomposition, with the singular-value
// cutoff max(m, n) * eps * sigma_max of torch.linalg.pinv's default.
void pinv_sym2(double a, double b, double c, double out[4]) {
  const double eps = 2.220446049250313e-16;
  const double mean = 0.5 * (a + c);
  const double half = 0.5 * (a - c);
  const double rad = std::sqrt(half * half + b * b);
  const double l1 = mean + rad, l2 = mean - rad;  // l1 >= l2
  const double smax = std::max(std::fabs(l1), std::fabs(l2));
  const double cut = 2.0 * eps * smax;
  const bool r1 = std::fabs(l1) > cut, r2 = std::fabs(l2) > cut;
  if (r1 && r2) {
    const double det = a * c - b * b;
    out[0] = c / det;
    out[1] = -b / det;
    out[2] = -b / det;
    out[3] = a / det;
    return;
  }
  out[0] = out[1] = out[2] = out[3] = 0.0;
  if (!r1) return;
  // rank one: pinv = v v^T / l1 with v the unit eigenvector of l1
  double vx, vy;
  if (std::fabs(b) > 0.0) {
    vx = l1 - c;
    vy = b;
  } else if (a >= c) {
    vx = 1.0;
    vy = 0.0;
  } else {
    vx = 0.0;
    vy = 1.0;
  }
  const double nv = std::sqrt(vx * vx + vy * vy);
  vx /= nv;
  vy /= nv;
  out[0] = vx * vx / l1;
  out[1] = vx * vy / l1;
  out[2] = vx * vy / l1;
  out[3] = vy * vy / l1;
}

template <class T>
int upload(std::string* err, T** dst, const std::vector<T>& src) {
  const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
  TDEM_CUDA_TRY(err, cudaMalloc(reinterpret_cast<void**>(dst), bytes));
  if (!src.empty()) TDEM_CUDA_TRY(err, cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return TDEM_OK;
}

}  // namespace

extern "C" {

int tdem_version(void) { return 1; }

int tdem_icedem_max_discs(void) { return tdem::icedem::kMaxDiscs; }

void tdem_icedem_destroy(tdem_icedem* h) {
  if (!h) return;
  cudaFree(h->bi);
  cudaFree(h->bj);
  cudaFree(h->inc_off);
  cudaFree(h->inc_bond);
  cudaFree(h->inc_other);
  cudaFree(h->bpair);
  cudaFree(h->rest);
  cudaFree(h->ref);
  cudaFree(h->pinv);
  cudaFree(h->hull);
  cudaFree(h->kcoef);
  cudaFree(h->ledger);
  cudaFree(h->energy);
  cudaFree(h->scratch);
  cudaFree(h->mbox);
  cudaFreeHost(h->mbox_host);
  cudaFreeHost(h->ledger_host);
  delete h;
}

int tdem_icedem_create(const tdem_icedem_config* cfg, const double* x0, tdem_icedem** out) {
  using namespace tdem::icedem;
  g_create_error.clear();
  std::string* err = &g_create_error;
  if (!cfg || !x0 || !out) return tdem::fail(err, TDEM_ERR_BADARG, "null argument");
  *out = nullptr;
  const int n = cfg->n;
  if (n < 2 || n > kMaxDiscs)
    return tdem::fail(err, TDEM_ERR_BADARG,
                      "reference mode supports 2.." + std::to_string(kMaxDiscs) + " discs, got " +
                          std::to_string(n));
  if (cfg->hull_vertices != 0 && (cfg->hull_vertices < 2 || cfg->hull_vertices > kMaxHull ||
                                  !cfg->hull_profile_host))
    return tdem::fail(err, TDEM_ERR_BADARG, "hull profile must have 2..64 vertices");
  if (!(cfg->dt > 0.0) || !(cfg->mass > 0.0) || !(cfg->radius > 0.0))
    return tdem::fail(err, TDEM_ERR_BADARG, "dt, mass and radius must be positive");

  auto* h = new tdem_icedem();
  h->n = n;
  h->npairs = (long long)n * (n - 1) / 2;
  Params& P = h->P;
  P.n = n;
  P.radius = cfg->radius;
  P.mass = cfg->mass;
  P.kb = cfg->bond_stiffness;
  P.kc = cfg->contact_stiffness;
  P.eps_t = cfg->breaking_strain;
  P.eps_s = cfg->shear_breaking_strain;
  P.cdamp = cfg->contact_damping;
  P.drag = cfg->drag;
  P.tool_radius = cfg->tool_radius;
  P.dt = cfg->dt;
  P.tool_start_x = cfg->tool_start[0];
  P.tool_start_y = cfg->tool_start[1];
  P.tool_vel_x = cfg->tool_velocity[0];
  P.tool_vel_y = cfg->tool_velocity[1];
  P.hull_m = cfg->hull_vertices;
  P.hull_start_x = cfg->hull_start[0];
  P.hull_start_y = cfg->hull_start[1];
  P.hull_vel_x = cfg->hull_velocity[0];
  P.hull_vel_y = cfg->hull_velocity[1];

  // Bonds: all pairs with |x0_j - x0_i| <= 2 r sqrt(2) (1 + 1e-10), pair order
  // (dem.py:116-129). Evaluated left to right like the reference expression.
  const double thr = ((2.0 * cfg->radius) * std::sqrt(2.0)) * (1.0 + 1e-10);
  std::vector<int> bi, bj;
  std::vector<long long> bpair;
  std::vector<double> rest;
  std::vector<double2> ref;
  long long p = 0;
  for (int i = 0; i < n; ++i) {
    for (int j = i + 1; j < n; ++j, ++p) {
      const double dx = x0[2 * j] - x0[2 * i], dy = x0[2 * j + 1] - x0[2 * i + 1];
      const double d = std::sqrt(std::fma(dy, dy, dx * dx));
      if (d <= thr) {
        bi.push_back(i);
        bj.push_back(j);
        bpair.push_back(p);
        rest.push_back(d);
        ref.push_back(make_double2(dx, dy));
      }
    }
  }
  const int nb = (int)bi.size();
  h->nbond = nb;
  P.nbond = nb;
  h->bpair_host = bpair;
  // Incidence lists in the reference's accumulation order: bonds where the
  // disc is i (ascending j), then bonds where it is j (ascending i).
  std::vector<std::vector<int>> first(n), second(n);
  for (int b = 0; b < nb; ++b) {
    first[bi[b]].push_back(b);
    second[bj[b]].push_back(b);
  }
  std::vector<int> inc_off(n + 1, 0), inc_bond, inc_other;
  std::vector<Mat2> pinv(n);
  for (int k = 0; k < n; ++k) {
    double c00 = 0.0, c01 = 0.0, c11 = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
      for (int b : (pass == 0 ? first[k] : second[k])) {
        inc_bond.push_back(b);
        inc_other.push_back(pass == 0 ? bj[b] : bi[b]);
        c00 += ref[b].x * ref[b].x;
        c01 += ref[b].x * ref[b].y;
        c11 += ref[b].y * ref[b].y;
      }
    }
    inc_off[k + 1] = (int)inc_bond.size();
    double q[4];
    pinv_sym2(c00, c01, c11, q);
    pinv[k] = Mat2{q[0], q[1], q[2], q[3]};
  }
  std::vector<double2> hull;
  for (int m = 0; m < cfg->hull_vertices; ++m)
    hull.push_back(make_double2(cfg->hull_profile_host[2 * m], cfg->hull_profile_host[2 * m + 1]));

  int rc = TDEM_OK;
  if ((rc = upload(err, &h->bi, bi)) || (rc = upload(err, &h->bj, bj)) ||
      (rc = upload(err, &h->bpair, bpair)) || (rc = upload(err, &h->rest, rest)) ||
      (rc = upload(err, &h->ref, ref)) || (rc = upload(err, &h->inc_off, inc_off)) ||
      (rc = upload(err, &h->inc_bond, inc_bond)) || (rc = upload(err, &h->inc_other, inc_other)) ||
      (rc = upload(err, &h->pinv, pinv)) || (rc = upload(err, &h->hull, hull))) {
    tdem_icedem_destroy(h);
    return rc;
  }
  std::vector<double> led(TDEM_L_COUNT, 0.0);
  led[TDEM_L_MIN_BREAK_MARGIN] = 1e300;
  if ((rc = upload(err, &h->ledger, led))) {
    tdem_icedem_destroy(h);
    return rc;
  }
  cudaError_t e = cudaMalloc(&h->mbox, sizeof(Mailbox));
  if (e == cudaSuccess) e = cudaMalloc(&h->energy, 5 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->scratch, (kMaxDiscs + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->mbox, 0, sizeof(Mailbox));
  if (e == cudaSuccess) e = cudaMallocHost(&h->mbox_host, sizeof(Mailbox));
  if (e == cudaSuccess) e = cudaMallocHost(&h->ledger_host, TDEM_L_COUNT * sizeof(double));
  if (e != cudaSuccess) {
    tdem_icedem_destroy(h);
    return tdem::fail(err, TDEM_ERR_CUDA, std::string("allocation: ") + cudaGetErrorString(e));
  }
  // One thread per disc (rounded to a warp), at most 512.
  h->threads = std::min(512, ((n + 31) / 32) * 32);
  const int nwarp = h->threads / 32;
  h->smem = (size_t)n * (16 + 16 + 16 + 8) + (size_t)(n + (n & 1)) * 8 + (size_t)12 * nwarp * 8 + 64;
  e = cudaFuncSetAttribute(icedem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem);
  if (e != cudaSuccess) {
    tdem_icedem_destroy(h);
    return tdem::fail(err, TDEM_ERR_CUDA, std::string("smem attribute: ") + cudaGetErrorString(e));
  }
  *out = h;
  return TDEM_OK;
}

int tdem_icedem_num_bonds(const tdem_icedem* h) { return h ? h->nbond : -1; }

int tdem_icedem_set_bond_stiffness(tdem_icedem* h, const double* k_host, int count) {
  if (!h || !k_host) return TDEM_ERR_BADARG;
  if (count != h->nbond)
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "per-bond stiffness count must equal the number of bonds");
  for (int b = 0; b < count; ++b)
    if (!(std::isfinite(k_host[b]) && k_host[b] > 0.0 && k_host[b] <= h->P.kb))
      return tdem::fail(&h->err, TDEM_ERR_BADARG,
                        "per-bond stiffness must be finite, positive and at most the config's bond stiffness");
  std::vector<double> k(k_host, k_host + count);
  if (h->kcoef) {
    cudaFree(h->kcoef);
    h->kcoef = nullptr;
  }
  return upload(&h->err, &h->kcoef, k);
}

int tdem_icedem_bond_pairs(const tdem_icedem* h, int64_t* out) {
  if (!h || !out) return TDEM_ERR_BADARG;
  std::memcpy(out, h->bpair_host.data(), h->bpair_host.size() * sizeof(int64_t));
  return TDEM_OK;
}

static int launch(tdem_icedem* h, const tdem_icedem_state* st, const double* loads, int mode,
                  int n_steps, double time, double* out_force, double* out_reaction, void* stream) {
  using namespace tdem::icedem;
  if (!st || !st->positions || !st->velocities || !st->initial_positions || !st->fixed ||
      !st->alive || !st->failure_mode || !st->failure_time_s || !st->failure_extension_m ||
      !st->failure_energy_J)
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "state pointer missing");
  Topo T{h->bi, h->bj, h->bpair, h->rest, h->ref, h->inc_off, h->inc_bond, h->inc_other, h->pinv, h->hull,
         h->kcoef};
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  icedem_kernel<<<1, h->threads, h->smem, s>>>(h->P, T, *st, reinterpret_cast<const double2*>(loads),
                                               mode, n_steps, time,
                                               reinterpret_cast<double2*>(out_force), out_reaction,
                                               h->ledger, h->mbox);
  TDEM_CUDA_TRY(&h->err, cudaGetLastError());
  return TDEM_OK;
}

int tdem_icedem_forces(tdem_icedem* h, const tdem_icedem_state* st, const double* loads, double time,
                       double* out_force, double* out_reaction, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  if (!out_force || !out_reaction) return tdem::fail(&h->err, TDEM_ERR_BADARG, "output pointer missing");
  return launch(h, st, loads, 1, 1, time, out_force, out_reaction, stream);
}

int tdem_icedem_step(tdem_icedem* h, const tdem_icedem_state* st, const double* loads, int n_steps,
                     double time, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  if (n_steps < 1) return tdem::fail(&h->err, TDEM_ERR_BADARG, "n_steps must be >= 1");
  int rc = launch(h, st, loads, 0, n_steps, time, nullptr, nullptr, stream);
  if (rc) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(h->mbox_host, h->mbox, sizeof(*h->mbox), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  if (h->mbox_host->status == TDEM_ERR_NONFINITE)
    return tdem::fail(&h->err, TDEM_ERR_NONFINITE,
                      "Non-finite simulation state; reduce dt (after step " +
                          std::to_string(h->mbox_host->steps_done) + " of the block)");
  return TDEM_OK;
}

int tdem_icedem_steps_done(const tdem_icedem* h) { return h ? h->mbox_host->steps_done : -1; }

int tdem_icedem_fragments(tdem_icedem* h, const void* alive, int32_t* labels_host, void* stream) {
  using namespace tdem::icedem;
  if (!h) return TDEM_ERR_BADARG;
  if (!alive || !labels_host) return tdem::fail(&h->err, TDEM_ERR_BADARG, "null argument");
  Topo T{h->bi, h->bj, h->bpair, h->rest, h->ref, h->inc_off, h->inc_bond, h->inc_other, h->pinv, h->hull,
         h->kcoef};
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int* dlabel = reinterpret_cast<int*>(h->scratch);
  int* drounds = dlabel + kMaxDiscs;
  icedem_fragment_kernel<<<1, h->threads, (size_t)h->n * sizeof(int), s>>>(h->P, T, static_cast<const bool*>(alive),
                                                                          dlabel, drounds);
  TDEM_CUDA_TRY(&h->err, cudaGetLastError());
  int rounds = 0;
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(labels_host, dlabel, (size_t)h->n * sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(&rounds, drounds, sizeof(int), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  if (rounds < 0) return tdem::fail(&h->err, TDEM_ERR_CUDA, "fragment labelling did not converge");
  return TDEM_OK;
}

int tdem_icedem_energy(tdem_icedem* h, const double* positions, const double* velocities, const void* alive,
                       double time, double* out_host, void* stream) {
  using namespace tdem::icedem;
  if (!h) return TDEM_ERR_BADARG;
  if (!positions || !velocities || !alive || !out_host)
    return tdem::fail(&h->err, TDEM_ERR_BADARG, "null argument");
  Topo T{h->bi, h->bj, h->bpair, h->rest, h->ref, h->inc_off, h->inc_bond, h->inc_other, h->pinv, h->hull,
         h->kcoef};
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  icedem_energy_kernel<<<1, h->threads, 0, s>>>(h->P, T, reinterpret_cast<const double2*>(positions),
                                                reinterpret_cast<const double2*>(velocities),
                                                static_cast<const bool*>(alive), time, h->energy);
  TDEM_CUDA_TRY(&h->err, cudaGetLastError());
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(out_host, h->energy, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  return TDEM_OK;
}



int tdem_icedem_read_ledger(tdem_icedem* h, double* out, int count, void* stream) {
  if (!h || !out || count < 0 || count > TDEM_L_COUNT) return TDEM_ERR_BADARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(h->ledger_host, h->ledger, TDEM_L_COUNT * sizeof(double),
                                         cudaMemcpyDeviceToHost, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  std::memcpy(out, h->ledger_host, count * sizeof(double));
  return TDEM_OK;
}

int tdem_icedem_ledger_to_device(tdem_icedem* h, double* out_device, void* stream) {
  if (!h || !out_device) return TDEM_ERR_BADARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(out_device, h->ledger, TDEM_L_COUNT * sizeof(double),
                                         cudaMemcpyDeviceToDevice, s));
  return TDEM_OK;
}

int tdem_icedem_write_ledger(tdem_icedem* h, const double* in, int count, void* stream) {
  if (!h || !in || count < 0 || count > TDEM_L_COUNT) return TDEM_ERR_BADARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  std::memcpy(h->ledger_host, in, count * sizeof(double));
  TDEM_CUDA_TRY(&h->err, cudaMemcpyAsync(h->ledger, h->ledger_host, count * sizeof(double),
                                         cudaMemcpyHostToDevice, s));
  TDEM_CUDA_TRY(&h->err, cudaStreamSynchronize(s));
  return TDEM_OK;
}

int tdem_icedem_last_error(const tdem_icedem* h, char* buf, size_t len) {
  if (!buf || len == 0) return TDEM_ERR_BADARG;
  const std::string& e = h ? h->err : g_create_error;
  const size_t m = std::min(len - 1, e.size());
  std::memcpy(buf, e.data(), m);
  buf[m] = '\0';
  return TDEM_OK;
}

}  // extern "C"
