// Batched ragged engine: many independent 2-D Hertz-Mindlin / bonded-disc
// solves of uneven sizes packed into one sorted SoA and advanced together by
// one persistent step kernel per step, inside the same conditional CUDA graph
// loop as the single-solve engine.
//
// Layout. Every instance owns a contiguous range of cell keys
// (key = key_off + cy * ncx + cx over its own grid), so after the cell sort
// its particles form one contiguous range of the sorted arrays. That range is
// cut into 32-particle tiles; a tile never straddles two instances. One warp
// processes one tile with the instance's parameters (copied once into shared
// memory), so the per-contact code is the single-solve engine's, unchanged.
//
// Ledger. Each tile writes one row of partial sums; the warp that finishes
// an instance's last tile (a per-instance ticket) sums the instance's rows in
// tile order. Results therefore do not depend on which other instances share
// the batch, nor on the grid shape, and carry no float atomics.
//
// Admission and retirement happen between step blocks. A new instance is
// appended behind the live particles and joins at the next rebuild; a retired
// one takes the dead key at the next rebuild and falls off the end of the
// sorted arrays. Instance slots and key ranges are reused only after that
// compaction.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "hm2d_dev.cuh"

namespace tdem {
namespace hm {

// ---------------------------------------------------------------------------
// Rebuild additions (every kernel a no-op unless ctl->rebuild_pending)
// ---------------------------------------------------------------------------
static __global__ void batch_begin_kernel(Ctl* ctl) {
  if (ctl->rebuild_pending) ctl->n_old = ctl->n_live;
}

// Live particles after the sort: everything before the dead key.
static __global__ void batch_count_kernel(Ctl* ctl, const int* cell_start) {
  if (ctl->rebuild_pending) ctl->n_live = cell_start[ctl->key_hi];
}

// Sorted range and first tile of every live instance slot (one block). Tiles
// are numbered kind-major: first the instances without bonds or indenter (run
// by the granular kernel build), then the others. ifirst[pass * slots + s] is
// slot s's first tile in its pass (non-decreasing over the whole array).
template <class T>
__global__ void batch_tiles_count_kernel(Bufs<T> B, int slots) {
  Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  int carry = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int c0 = 0; c0 < slots; c0 += kScanChunk) {
      const int base = c0 + threadIdx.x * kScanItems;
      int st[kScanItems], en[kScanItems], nt[kScanItems];
      bool mine[kScanItems];
      int local = 0;
      for (int k = 0; k < kScanItems; ++k) {
        const int s = base + k;
        st[k] = en[k] = nt[k] = 0;
        mine[k] = false;
        if (s < slots && (B.istate[s] & kInstAlive)) {
          const Params<T>& Q = B.iparams[s];
          mine[k] = (Q.feat != 0) == (pass == 1);
          if (mine[k]) {
            st[k] = B.cell_start[Q.key_off];
            en[k] = B.cell_start[Q.key_off + Q.ncx * Q.ncy];
            nt[k] = (en[k] - st[k] + kTile - 1) / kTile;
          }
        } else if (s < slots && pass == 0) {
          mine[k] = true;  // dead or free slot: an empty range
        }
        local += nt[k];
      }
      int total;
      int run = carry + block_exclusive_scan(local, &total);
      for (int k = 0; k < kScanItems; ++k) {
        const int s = base + k;
        if (s < slots) {
          B.ifirst[pass * slots + s] = run;
          if (mine[k]) B.irange[s] = make_int4(st[k], en[k], run, nt[k]);
        }
        run += nt[k];
      }
      carry += total;
    }
    if (pass == 0 && threadIdx.x == 0) ctl->ntiles_plain = carry;
  }
  if (threadIdx.x == 0) ctl->ntiles = carry;
}

// Tile table: tile t belongs to the last entry of ifirst that is <= t.
template <class T>
__global__ void batch_tiles_fill_kernel(Bufs<T> B, int slots) {
  const Ctl* ctl = B.ctl;
  if (!ctl->rebuild_pending) return;
  const int nt = ctl->ntiles;
  const int m = 2 * slots;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    int lo = 0, hi = m;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (B.ifirst[mid] <= t)
        lo = mid + 1;
      else
        hi = mid;
    }
    const int s = (lo - 1) % slots;  // ifirst[0] == 0 <= t, so lo >= 1
    const int4 r = B.irange[s];
    const int first = r.x + (t - r.z) * kTile;
    B.tiles[t] = make_int4(s, first, min(kTile, r.y - first), 0);
  }
}

// ---------------------------------------------------------------------------
// The batched step kernel (MODE kBatch) and read-back (MODE kPeek: only the
// tiles of instances flagged kInstPeek). Persistent: each warp strides over
// tiles with the next tile's loads in flight.
// ---------------------------------------------------------------------------
constexpr unsigned kFull = 0xffffffffu;

template <class T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(kFull, x, off);
  return x;
}

// PART 0: every tile (read-back); 1: the granular instances' tiles, granular
// code, no step bookkeeping; 2: the other tiles, full code, and the step
// bookkeeping (it runs after part 1 in the same stream). CHUNK: tiles per
// grab from the step kernel's work counter.
template <class T, int MODE, int BLOCK, int MINB, int PART, int CHUNK = 8>
__global__ void __launch_bounds__(BLOCK, MINB)
    batch_kernel(Bufs<T> B, cudaGraphConditionalHandle h_rebuild, cudaGraphConditionalHandle h_loop,
                 int use_cond, int rebuild_every) {
  static_assert(MODE == kBatch || MODE == kPeek, "batched modes only");
  static_assert((MODE == kPeek) == (PART == 0), "read-back covers every tile; steps run in two parts");
  constexpr bool FEAT = PART != 1;
  constexpr int NW = BLOCK / 32;
  constexpr int PW = (int)(sizeof(Params<T>) / 4);
  static_assert(sizeof(Params<T>) % 4 == 0, "Params copied as 32-bit words");
  __shared__ alignas(16) Params<T> s_par[NW];
  __shared__ unsigned s_warps_done;
  Ctl* ctl = B.ctl;
  const int sp = ctl->sp, lp = ctl->lp;
  const long long eval = ctl->evals;
  const int tbeg = PART == 2 ? ctl->ntiles_plain : 0;
  const int ntiles = PART == 1 ? ctl->ntiles_plain : ctl->ntiles;
  // written only by the last warp of this kernel, after every block read them
  const float disp0 = ctl->disp;
  const int since0 = ctl->since;
  const long long target = ctl->target;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nwarps = gridDim.x * NW;
  if (threadIdx.x == 0) s_warps_done = 0u;
  __syncthreads();
  Params<T>& Q = s_par[wib];
  float vmax = 0.0f;  // max over this thread's tiles of (|v| dt / rebuild displacement)^2
  const V4<T>* __restrict__ pos = B.pos[sp];
  const V4<T>* __restrict__ vel = B.vel[sp];
  const uint4* __restrict__ head = B.head[lp];
  // Tiles are handed out in chunks of CHUNK consecutive tiles (step kernel:
  // from an atomic counter, so fast and slow tiles balance; read-back: one
  // static chunk per warp). Consecutive tiles mostly belong to one instance,
  // so its parameters are copied once and its ticket is taken once per
  // (chunk, instance) segment. Rows stay per tile: the instance sums do not
  // depend on which warp took which tile. A warp holds two chunks at a time
  // (the one it works on and the next), so small batches balance only with
  // short chunks; large ones take long chunks, which keeps the atomics few.
  const int per = (MODE == kBatch) ? CHUNK : (ntiles + nwarps - 1) / nwarps;
  const int gw = blockIdx.x * NW + wib;
  int grabs = 0;
  auto grab = [&]() -> int {
    if (MODE == kPeek) return (grabs++ == 0) ? (int)min((long long)gw * per, (long long)ntiles) : ntiles;
    int b = 0;
    if (lane == 0) b = tbeg + atomicAdd(PART == 1 ? &ctl->tile_next : &ctl->tile_next2, CHUNK);
    return __shfl_sync(kFull, b, 0);
  };
  int t = grab();
  int tend = min(t + per, ntiles);
  int nb = (t < ntiles) ? grab() : ntiles;  // start of the chunk after this one
  int4 d = make_int4(0, 0, 0, 0);
  V4<T> p{}, v{};
  uint4 hd = make_uint4(0u, 0u, 0u, 0u);
  // the position remainders travel with the own state (FP32 batches that keep them)
  const float2* __restrict__ prem = B.prem[lp];
  float2 r{0.0f, 0.0f};
  if (t < tend) {
    d = B.tiles[t];
    if (lane < d.z) {
      p = pos[d.y + lane];
      v = vel[d.y + lane];
      hd = head[d.y + lane];
      if (prem) r = prem[d.y + lane];
    }
  }
  bool frozen = false;  // the open segment's instance has taken all its steps
  int seg_k = -1;  // instance of the open segment
  int seg_n = 0;   // tiles of the open segment processed by this warp
  bool run = false;
  long long le = 0;  // the instance's own evaluation index
  int primed = 0;
  // Close a segment: take the instance's ticket for its tiles; the warp that
  // completes the instance sums the instance's rows in tile order.
  auto flush = [&]() {
    if (seg_n == 0) return;
    const int k = seg_k;
    unsigned last = 0u;
    if (lane == 0) {
      __threadfence();
      const unsigned nt = (unsigned)B.irange[k].w;
      last = (atomicAdd(&B.iticket[k], (unsigned)seg_n) + (unsigned)seg_n == nt) ? 1u : 0u;
    }
    last = __shfl_sync(kFull, last, 0);
    seg_n = 0;
    if (!last) return;
    __threadfence();
    const int4 r = B.irange[k];
    constexpr int NV = (MODE == kBatch) ? 5 : 9;
    double s[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) s[c] = 0.0;
    for (int tt = r.z + lane; tt < r.z + r.w; tt += 32) {
      const double* rr = B.tpart + (size_t)tt * kTileVals;
#pragma unroll
      for (int c = 0; c < NV; ++c) s[c] += __ldcg(rr + c);
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) s[c] = warp_sum<double>(s[c]);
    if (lane == 0) {
      double* led = B.iled + (size_t)k * kInstLedger;
      if (MODE == kBatch) {
        led[0] += s[0];                                                // dissipated
        led[1] += s[1];                                                // fracture release
        led[2] += (double)Q.dt * (s[2] * Q.ind_vx + s[3] * Q.ind_vy);  // tool work
        led[3] += s[4];                                                // bonds broken
        led[4] = -s[2];                                                // reaction on the indenter
        led[5] = -s[3];
        const double R = sqrt(s[2] * s[2] + s[3] * s[3]);
        if (R > led[6]) {
          led[6] = R;
          led[7] = (double)le;
        }
        led[8] = (double)(le + 1);  // evaluations committed
      } else {
#pragma unroll
        for (int c = 0; c < 9; ++c) led[9 + c] = s[c];
      }
      B.iticket[k] = 0u;
    }
  };
  while (t < tend) {
    int tn = t + 1, tnend = tend;
    bool next_chunk = false;
    if (tn >= tend) {
      tn = nb;
      tnend = min(nb + per, ntiles);
      next_chunk = true;
    }
    int4 dn = make_int4(0, 0, 0, 0);
    V4<T> pn{}, vn{};
    uint4 hn = make_uint4(0u, 0u, 0u, 0u);
    float2 rn{0.0f, 0.0f};
    if (tn < tnend) {
      dn = B.tiles[tn];
      if (lane < dn.z) {
        pn = pos[dn.y + lane];
        vn = vel[dn.y + lane];
        hn = head[dn.y + lane];
        if (prem) rn = prem[dn.y + lane];
      }
    }
    const int k = d.x;
    if (k != seg_k) {
      flush();
      seg_k = k;
      const int st = B.istate[k];
      run = (MODE == kPeek) ? (st & kInstPeek) != 0 : (st & kInstAlive) != 0;
      if (run) {
        __syncwarp();
        const unsigned* src = reinterpret_cast<const unsigned*>(B.iparams + k);
        unsigned* dst = reinterpret_cast<unsigned*>(&Q);
        for (int w = lane; w < PW; w += 32) dst[w] = src[w];
        __syncwarp();
        le = eval - Q.eval0;
        primed = le > 0 ? 1 : 0;
        // quarantine: an instance with a non-finite state, an escaped particle or
        // an overflowed neighbour list stops (its status is reported), so it can
        // neither slow the shared rebuild trigger nor spread garbage
        const int bad = (st | (st >> kInstRebuildShift)) & (kStatusNonfinite | kStatusEscaped | kStatusCapacity);
        frozen = MODE == kBatch && (le >= Q.stop || bad != 0);
      }
    }
    if (run && frozen) {
      // carry the state over unchanged (no forces, no ledger, no ticket)
      if (lane < d.z) {
        B.pos[sp ^ 1][d.y + lane] = p;
        B.vel[sp ^ 1][d.y + lane] = v;
      }
    } else if (run) {
      ThreadLedger<T> L;
      if (lane < d.z) process_particle<T, MODE, FEAT>(Q, B, sp, lp, d.y + lane, p, v, hd, primed, le, L, &r);
      double* row = B.tpart + (size_t)t * kTileVals;
      if (MODE == kBatch) {
        const float f = (float)Q.dt / Q.rebuild_disp;
        vmax = fmaxf(vmax, L.vmax2 * f * f);
        const T wd = warp_sum<T>(L.diss);
        T wf = T(0), wix = T(0), wiy = T(0);
        int wb = 0;
        if (__any_sync(kFull, L.frac != T(0) || L.ifx != T(0) || L.ify != T(0) || L.broke != 0)) {
          wf = warp_sum<T>(L.frac);
          wix = warp_sum<T>(L.ifx);
          wiy = warp_sum<T>(L.ify);
          wb = warp_sum<int>(L.broke);
        }
        const bool bad = __any_sync(kFull, L.bad);
        if (lane == 0) {
          row[0] = (double)wd;
          row[1] = (double)wf;
          row[2] = (double)wix;
          row[3] = (double)wiy;
          row[4] = (double)wb;
          if (bad) atomicOr(&B.istate[k], (int)kStatusNonfinite);
        }
      } else {
        const double a0 = warp_sum<double>(L.ke), a1 = warp_sum<double>(L.pe);
        const T a2 = warp_sum<T>(L.un), a3 = warp_sum<T>(L.ut);
        const T a4 = warp_sum<T>(primed ? L.diss : T(0));
        const T a5 = warp_sum<T>(L.ub), a6 = warp_sum<T>(L.frac);
        const T a7 = warp_sum<T>((L.ifx * (T)Q.ind_vx + L.ify * (T)Q.ind_vy) * Q.dt);
        const T a8 = warp_sum<T>((T)L.broke);
        if (lane == 0) {
          row[0] = a0;
          row[1] = a1;
          row[2] = (double)a2;
          row[3] = (double)a3;
          row[4] = (double)a4;
          row[5] = (double)a5;
          row[6] = (double)a6;
          row[7] = (double)a7;
          row[8] = (double)a8;
        }
      }
      ++seg_n;
    }
    t = tn;
    tend = tnend;
    d = dn;
    p = pn;
    v = vn;
    hd = hn;
    r = rn;
    if (next_chunk && t < tend) nb = grab();
  }
  flush();
  if constexpr (MODE == kBatch) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(kFull, vmax, off));
    if (lane != 0) return;
    const unsigned bits = __float_as_uint(vmax);
    if (bits > *reinterpret_cast<volatile unsigned*>(&ctl->vmax2_bits)) atomicMax(&ctl->vmax2_bits, bits);
    if (PART == 1) return;  // the second launch does the step bookkeeping
    __threadfence();
    const unsigned mine = atomicAdd(&s_warps_done, 1u);
    if (mine != NW - 1) return;
    const unsigned tk = atomicAdd(&ctl->ticket, 1u);
    if (tk != gridDim.x - 1) return;
    // last warp of the grid: step bookkeeping and the graph's conditions. The
    // speed bound is read by an atomic at L2, issued only after the ticket's
    // value was tested, so no fence is needed here.
    const float vm = sqrtf(__uint_as_float(atomicExch(&ctl->vmax2_bits, 0u)));
    ctl->ticket = 0;
    ctl->tile_next = 0;
    ctl->tile_next2 = 0;
    ctl->sp = sp ^ 1;
    ctl->evals = eval + 1;
    const float disp = disp0 + vm;  // in units of each instance's allowed displacement
    ctl->disp = disp;
    const int since = since0 + 1;
    ctl->since = since;
    const int rebuild = (disp > 1.0f || (rebuild_every > 0 && since >= rebuild_every)) ? 1 : 0;
    ctl->rebuild_pending = rebuild;
    const int keep_going = eval + 1 < target;
    if (use_cond & 1) cudaGraphSetConditional(h_rebuild, (unsigned)rebuild);
    if (use_cond & 2) cudaGraphSetConditional(h_loop, (unsigned)keep_going);
  }
}

// ---------------------------------------------------------------------------
// Admission, read-back and retirement kernels
// ---------------------------------------------------------------------------

// Append m particles of instance `slot` behind the live ones (host layout,
// FP64, instance-local order), in the current buffers.
template <class T>
__global__ void batch_append_kernel(Params<T> Q, Bufs<T> B, int slot, int m, const double* pos, const double* vel,
                                    const double* omega, const double* radius, const double* mass,
                                    const double* inertia) {
  const Ctl* ctl = B.ctl;
  const int base = ctl->n_live;
  const int sp = ctl->sp, lp = ctl->lp;
  const size_t n = (size_t)Q.n;
  const double c = (double)Q.cell;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const int i = base + j;
    const double x = pos[2 * j], y = pos[2 * j + 1];
    double fx = floor(x / c), fy = floor(y / c);
    if (!(fx == fx)) fx = 0.0;
    if (!(fy == fy)) fy = 0.0;
    const int cx = (int)fmin(fmax(fx, 0.0), (double)(Q.ncx - 1));
    const int cy = (int)fmin(fmax(fy, 0.0), (double)(Q.ncy - 1));
    const double r = radius[j], ms = mass[j];
    const bool clamped = isinf(ms) && ms > 0.0;  // infinite mass: a clamped disc
    const double ox = x - cx * c, oy = y - cy * c;
    B.pos[sp][i] = V4<T>{(T)ox, (T)oy, (T)r, cell_to_lane(cx | (cy << 16), T(0))};
    if (sizeof(T) == 4 && Q.prem)
      B.prem[lp][i] = make_float2((float)(ox - (double)(T)ox), (float)(oy - (double)(T)oy));
    B.vel[sp][i] = clamped ? V4<T>{T(0), T(0), T(0), T(0)}
                           : V4<T>{(T)vel[2 * j], (T)vel[2 * j + 1], (T)omega[j], (T)(1.0 / ms)};
    if (B.bcnt[lp]) B.bcnt[lp][i] = 0;
    B.head[lp][i] = make_uint4(0u, 0u, 0u, 0u);
    B.orig[lp][i] = j;
    B.inst[lp][i] = slot;
    for (int w = 0; w < 4; ++w) B.whist[lp][(size_t)w * n + i] = V2<T>{T(0), T(0)};
    const double want = ms * r * r / (double)Q.kinv;
    if (!clamped && !(fabs(inertia[j] - want) <= 1e-6 * fabs(want))) atomicOr(&B.istate[slot], (int)kStatusInertia);
  }
}

// Bond slots of the appended particles: part_local / strength are [BMAX * m]
// slot-major in instance-local ids (-1: no bond in that slot).
template <class T>
__global__ void batch_bond_init_kernel(Params<T> Q, Bufs<T> B, int m, const int* part_local, const float* strength) {
  const Ctl* ctl = B.ctl;
  const int base = ctl->n_live;
  const int sp = ctl->sp, lp = ctl->lp;
  const size_t n = (size_t)Q.n;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const int p = base + j;
    const V4<T> a = B.pos[sp][p];
    int bc = 0;
    T c00 = 0, c01 = 0, c11 = 0;
    for (int s = 0; s < Q.BMAX; ++s) {
      const int ql = part_local[(size_t)s * m + j];
      if (ql < 0) break;
      const int q = base + ql;
      const V2<T> r = cell_delta<T>(Q, a, B.pos[sp][q]);
      const size_t k = (size_t)s * n + p;
      B.bpart[lp][k] = (unsigned)q;
      B.bref[lp][k] = r;
      B.bstr[lp][k] = (T)strength[(size_t)s * m + j];
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
}

template <class T>
__global__ void batch_set_params_kernel(Params<T>* dst, Params<T> v) {
  *dst = v;
}

// Make an appended instance live: count its particles, clear its ledger row
// and ticket, move the dead key, and ask for the rebuild that sorts it in.
static __global__ void batch_admit_kernel(Ctl* ctl, int* istate, unsigned* iticket, double* iled, int slot, int m,
                                          int key_hi) {
  ctl->n_live += m;
  ctl->key_hi = key_hi;
  ctl->rebuild_pending = 1;
  istate[slot] = kInstAlive;
  iticket[slot] = 0u;
  for (int k = 0; k < kInstLedger; ++k) iled[(size_t)slot * kInstLedger + k] = 0.0;
}

static __global__ void batch_state_kernel(int* istate, int slot, int set, int clear) {
  istate[slot] = (istate[slot] & ~clear) | set;
}

static __global__ void batch_key_hi_kernel(Ctl* ctl, int key_hi) { ctl->key_hi = key_hi; }

static __global__ void batch_state_list_kernel(int* istate, const int* ids, int count, int set, int clear) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count; j += gridDim.x * blockDim.x)
    istate[ids[j]] = (istate[ids[j]] & ~clear) | set;
}

// Integer-time state of one instance in its local order (after a kPeek pass).
template <class T>
__global__ void batch_unpack_kernel(Params<T> Q, Bufs<T> B, int slot, int m, double* out) {
  const Ctl* ctl = B.ctl;
  const int sp = ctl->sp, lp = ctl->lp;
  const int4 r = B.irange[slot];
  double* pos = out;
  double* vel = out + 2 * (size_t)m;
  double* omega = out + 4 * (size_t)m;
  double* force = out + 5 * (size_t)m;
  double* torque = out + 7 * (size_t)m;
  const double cl = (double)Q.cell;
  for (int p = r.x + blockIdx.x * blockDim.x + threadIdx.x; p < r.y; p += gridDim.x * blockDim.x) {
    const int o = B.orig[lp][p];
    if (o < 0 || o >= m) continue;
    const V4<T> q = B.pos[sp][p];
    const int c = lane_to_cell(q.w);
    const float2 rm = (sizeof(T) == 4 && Q.prem) ? B.prem[lp][p] : make_float2(0.0f, 0.0f);
    pos[2 * o] = (double)(c & 0xFFFF) * cl + (double)q.x + (double)rm.x;
    pos[2 * o + 1] = (double)(c >> 16) * cl + (double)q.y + (double)rm.y;
    const V4<T> v = B.peek_vel[p];
    vel[2 * o] = (double)v.x;
    vel[2 * o + 1] = (double)v.y;
    omega[o] = (double)v.z;
    const V4<T> f = B.peek_force[p];
    force[2 * o] = (double)f.x;
    force[2 * o + 1] = (double)f.y;
    torque[o] = (double)f.z;
  }
}

// Bond states of one instance as local ids (lo, hi) with mode and break evaluation.
template <class T>
__global__ void batch_bonds_out_kernel(Params<T> Q, Bufs<T> B, int slot, int* pairs, int* state, long long capacity,
                                       unsigned long long* count) {
  const Ctl* ctl = B.ctl;
  const int lp = ctl->lp;
  const int4 r = B.irange[slot];
  const size_t n = (size_t)Q.n;
  for (int p = r.x + blockIdx.x * blockDim.x + threadIdx.x; p < r.y; p += gridDim.x * blockDim.x) {
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
      state[2 * e] = (w & kBondBroken) ? (int)((w >> kBondModeShift) & 3u) : 0;
      state[2 * e + 1] = B.bfail[lp][k];
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

// Step-kernel shapes: block size, CTAs per SM and tiles per grab. 4 and 5 are
// 1 and 3 with 2-tile grabs, for batches with few tiles per warp.
constexpr int kBatchVariants = 6;
inline int bvariant_block(int v) { return (v == 0 || v == 2) ? 256 : 128; }

template <class T>
using BatchFn = void (*)(Bufs<T>, cudaGraphConditionalHandle, cudaGraphConditionalHandle, int, int);

template <class T, int PART>
BatchFn<T> batch_fn_part(int variant) {
  switch (variant) {
    case 1: return &batch_kernel<T, kBatch, 128, 4, PART>;
    case 2: return &batch_kernel<T, kBatch, 256, 3, PART>;
    case 3: return &batch_kernel<T, kBatch, 128, 6, PART>;
    case 4: return &batch_kernel<T, kBatch, 128, 4, PART, 2>;
    case 5: return &batch_kernel<T, kBatch, 128, 6, PART, 2>;
    default: return &batch_kernel<T, kBatch, 256, 2, PART>;
  }
}

// part 0: read-back over every tile; 1 / 2: the two launches of a step
template <class T>
BatchFn<T> batch_fn(int variant, int part) {
  if (part == 0) return &batch_kernel<T, kPeek, 256, 2, 0>;
  return part == 1 ? batch_fn_part<T, 1>(variant) : batch_fn_part<T, 2>(variant);
}

inline int bvariant_minb(int v) { return v == 0 ? 2 : (v == 1 || v == 4) ? 4 : v == 2 ? 3 : 6; }

// One device allocation, carved into 256-byte aligned arrays.
struct Arena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  template <class U>
  U* take(size_t count) {
    used = (used + 255) & ~size_t(255);
    U* p = reinterpret_cast<U*>(base ? base + used : nullptr);
    used += count * sizeof(U);
    return p;
  }
};

struct BatchBase {
  virtual ~BatchBase() = default;
  virtual int admit(const tdem_hm_config& c, const double* pos, const double* vel, const double* omega,
                    const double* radius, const double* mass, const double* inertia, const int* bonds,
                    const double* strength, long long nb, int* id, cudaStream_t s) = 0;
  virtual int step(long long n, cudaStream_t s) = 0;
  virtual int read(int id, double* pos, double* vel, double* omega, double* force, double* torque, double* ledger,
                   int count, cudaStream_t s) = 0;
  virtual int retire(int id, cudaStream_t s) = 0;
  virtual int set_steps(int id, long long steps, cudaStream_t s) = 0;
  virtual int read_ledgers(const int* ids, int count, double* out, cudaStream_t s) = 0;
  virtual int read_bonds(int id, int* pairs, int* state, long long cap, long long* count, cudaStream_t s) = 0;
  virtual int info(long long* out, int count, cudaStream_t s) = 0;
  virtual int set_variant(int v) = 0;
  virtual int get_variant() const = 0;
  virtual int autotune(int steps, cudaStream_t s, float* ms_out) = 0;
  virtual int use_graph(int on) = 0;
  std::string err;
};

template <class T>
struct Batch final : BatchBase {
  tdem_batch_config cfg{};
  Params<T> G{};  // n = particle capacity (the stride of slot-major arrays), W, BMAX
  Bufs<T> B{};
  Params<T>* iparams = nullptr;
  Arena arena;
  int slots = 0;
  int sms = 0;
  int variant = 0;
  bool graph_on = true, graph_failed = false;
  // host view of the instances
  struct Inst {
    int state = 0;  // 0 free, 1 live, 2 retired (waiting for the compaction rebuild)
    int n = 0;
    int key_off = 0, nkeys = 0;
    long long eval0 = 0;
    Params<T> par{};
  };
  std::vector<Inst> inst;
  std::vector<int> free_slots, pending_slots;
  std::map<int, int> free_keys;  // start -> length (unallocated key ranges)
  std::map<int, int> used_keys;  // start -> length (allocated, incl. pending)
  std::vector<std::pair<int, int>> pending_keys;
  long long occupied = 0;  // particles in the arrays, dead ones included
  long long live = 0;
  long long evals = 0;
  bool need_rebuild = false;
  int key_hi = 0;
  // staging
  double* stage_dev = nullptr;
  double* stage_host = nullptr;
  int* bpart_dev = nullptr;
  float* bstr_dev = nullptr;
  int* bpart_host = nullptr;
  float* bstr_host = nullptr;
  size_t stage_cap = 0;  // particles
  unsigned long long* count_dev = nullptr;
  unsigned long long* count_host = nullptr;
  Ctl* host_ctl = nullptr;
  double* host_led = nullptr;
  int* host_state = nullptr;
  int* list_dev = nullptr;
  int* list_host = nullptr;
  size_t list_cap = 0;
  std::vector<double> all_led;
  double* all_led_host = nullptr;
  int* all_state_host = nullptr;
  // graph
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t target_node = nullptr;
  cudaGraphConditionalHandle h_loop = 0, h_reb = 0;
  long long exec_target = -1;

  ~Batch() override {
    destroy_graphs();
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (arena.base) cudaFree(arena.base);
    if (stage_dev) cudaFree(stage_dev);
    if (bpart_dev) cudaFree(bpart_dev);
    if (bstr_dev) cudaFree(bstr_dev);
    if (stage_host) cudaFreeHost(stage_host);
    if (bpart_host) cudaFreeHost(bpart_host);
    if (bstr_host) cudaFreeHost(bstr_host);
    if (count_dev) cudaFree(count_dev);
    if (count_host) cudaFreeHost(count_host);
    if (host_ctl) cudaFreeHost(host_ctl);
    if (host_led) cudaFreeHost(host_led);
    if (host_state) cudaFreeHost(host_state);
    if (list_dev) cudaFree(list_dev);
    if (list_host) cudaFreeHost(list_host);
    if (all_led_host) cudaFreeHost(all_led_host);
    if (all_state_host) cudaFreeHost(all_state_host);
  }

  void destroy_graphs() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    exec_target = -1;
  }

  // Carve every array out of the arena (a null base only measures).
  void carve(Arena& a) {
    const size_t N = (size_t)cfg.particle_capacity;
    const size_t K = (size_t)cfg.key_capacity;
    const size_t W = (size_t)G.W;
    const size_t BM = (size_t)G.BMAX;
    const size_t tiles_cap = N / kTile + (size_t)slots + 1;
    for (int b = 0; b < 2; ++b) {
      B.pos[b] = a.take<V4<T>>(N);
      B.vel[b] = a.take<V4<T>>(N);
      B.head[b] = a.take<uint4>(N);
      B.nbr[b] = a.take<unsigned>(N * std::max<size_t>(W > 3 ? W - 3 : 1, 1));
      B.hist[b] = a.take<V2<T>>(N * W);
      B.orig[b] = a.take<int>(N);
      B.inst[b] = a.take<int>(N);
      B.whist[b] = a.take<V2<T>>(4 * N);
      B.prem[b] = (sizeof(T) == 4 && cfg.position_remainder) ? a.take<float2>(N) : nullptr;
      if (BM > 0) {
        B.bpart[b] = a.take<unsigned>(BM * N);
        B.bref[b] = a.take<V2<T>>(BM * N);
        B.bstr[b] = a.take<T>(BM * N);
        B.bus[b] = a.take<V2<T>>(BM * N);
        B.bfail[b] = a.take<int>(BM * N);
        B.bcnt[b] = a.take<int>(N);
        B.bpinv[b] = a.take<V4<T>>(N);
      }
    }
    B.cell_count = a.take<int>(K);
    B.cell_start = a.take<int>(K);
    B.cell_fill = a.take<int>(K);
    B.block_sums = a.take<int>((K + kScanChunk - 1) / kScanChunk + 1);
    B.perm = a.take<int>(N);
    B.invperm = a.take<int>(N);
    B.tmp_cell = a.take<int>(N);
    B.tmp_off = a.take<V2<T>>(N);
    B.tmp_key = a.take<int>(N);
    B.strain = a.take<T>(N);
    B.peek_vel = a.take<V4<T>>(N);
    B.peek_force = a.take<V4<T>>(N);
    B.ctl = a.take<Ctl>(1);
    iparams = a.take<Params<T>>((size_t)slots);
    B.iparams = iparams;
    B.istate = a.take<int>((size_t)slots);
    B.irange = a.take<int4>((size_t)slots);
    B.ifirst = a.take<int>(2 * (size_t)slots);
    B.iticket = a.take<unsigned>((size_t)slots);
    B.iled = a.take<double>((size_t)slots * kInstLedger);
    B.tiles = a.take<int4>(tiles_cap);
    B.tpart = a.take<double>(tiles_cap * kTileVals);
  }

  static int check_config(const tdem_batch_config& c, std::string& e) {
    if (c.precision != 32 && c.precision != 64) return tdem::fail(&e, TDEM_ERR_BADARG, "precision must be 32 or 64");
    if (c.max_neighbors < 1 || c.max_neighbors > kMaxSlots)
      return tdem::fail(&e, TDEM_ERR_BADARG, "max_neighbors must be in 1..24");
    if (c.max_bonds < 0 || c.max_bonds > kMaxBondSlots)
      return tdem::fail(&e, TDEM_ERR_BADARG, "max_bonds must be in 0..8");
    if (c.max_instances < 1 || c.max_instances > (1 << 20))
      return tdem::fail(&e, TDEM_ERR_BADARG, "max_instances must be in 1..1048576");
    if (c.particle_capacity < 32 || c.particle_capacity > (1ll << 29) - 64)
      return tdem::fail(&e, TDEM_ERR_BADARG, "particle_capacity must be in 32..2^29-64");
    if (c.key_capacity < 2 || c.key_capacity > (1ll << 31) - 1)
      return tdem::fail(&e, TDEM_ERR_BADARG, "key_capacity must be in 2..2^31-1");
    if (c.rebuild_every < 0) return tdem::fail(&e, TDEM_ERR_BADARG, "rebuild_every must be >= 0");
    if (c.position_remainder != 0 && c.position_remainder != 1)
      return tdem::fail(&e, TDEM_ERR_BADARG, "position_remainder must be 0 or 1");
    return TDEM_OK;
  }

  int init(const tdem_batch_config& c) {
    cfg = c;
    slots = c.max_instances;
    G.n = (int)c.particle_capacity;
    G.W = c.max_neighbors;
    G.BMAX = c.max_bonds;
    G.prem = (sizeof(T) == 4 && c.position_remainder) ? 1 : 0;
    int dev = 0;
    TDEM_CUDA_TRY(&err, cudaGetDevice(&dev));
    TDEM_CUDA_TRY(&err, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    Arena probe;
    carve(probe);
    arena.size = probe.used + 256;
    TDEM_CUDA_TRY(&err, cudaMalloc(&arena.base, arena.size));
    carve(arena);
    // zero what must start at zero: key counters, control block, instance words
    TDEM_CUDA_TRY(&err, cudaMemset(B.cell_count, 0, (size_t)cfg.key_capacity * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.cell_fill, 0, (size_t)cfg.key_capacity * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.ctl, 0, sizeof(Ctl)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.istate, 0, (size_t)slots * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.iticket, 0, (size_t)slots * sizeof(unsigned)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.iled, 0, (size_t)slots * kInstLedger * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMemset(B.irange, 0, (size_t)slots * sizeof(int4)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_ctl, sizeof(Ctl)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_led, kInstLedger * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&host_state, sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&count_dev, sizeof(unsigned long long)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&count_host, sizeof(unsigned long long)));
    TDEM_CUDA_TRY(&err, cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    TDEM_CUDA_TRY(&err, cudaDeviceSynchronize());
    inst.assign((size_t)slots, Inst{});
    for (int k = slots - 1; k >= 0; --k) free_slots.push_back(k);
    // the last key is kept back: it is the dead key when every other key is in use
    free_keys[0] = (int)(cfg.key_capacity - 1);
    key_hi = 0;
    return TDEM_OK;
  }

  // Grid of the per-particle / per-key rebuild kernels (grid-stride loops).
  unsigned grid_items(long long items) const {
    const long long want = (items + kThreads - 1) / kThreads;
    return (unsigned)std::max<long long>(1, std::min<long long>(want, (long long)sms * 8));
  }

  void launch_rebuild(cudaStream_t s) {
    const unsigned gn = grid_items(cfg.particle_capacity);
    const unsigned gk = grid_items(cfg.key_capacity);
    const unsigned sb = (unsigned)((cfg.key_capacity + kScanChunk - 1) / kScanChunk);
    batch_begin_kernel<<<1, 1, 0, s>>>(B.ctl);
    bin_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    scan_blocks_kernel<<<sb, kScanThreads, 0, s>>>(B.ctl, B.cell_count, B.cell_start, B.block_sums, -1);
    scan_top_kernel<<<1, kScanThreads, 0, s>>>(B.ctl, B.block_sums, -1);
    scan_add_kernel<<<sb, kScanThreads, 0, s>>>(B.ctl, B.cell_start, B.block_sums, -1);
    batch_count_kernel<<<1, 1, 0, s>>>(B.ctl, B.cell_start);
    scatter_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    cellsort_kernel<T, true><<<gk, kThreads, 0, s>>>(G, B);
    gather_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    bond_gather_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    build_nbr_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    link_kernel<T, true><<<gn, kThreads, 0, s>>>(G, B);
    batch_tiles_count_kernel<T><<<1, kScanThreads, 0, s>>>(B, slots);
    batch_tiles_fill_kernel<T><<<grid_items(cfg.particle_capacity / kTile + slots), kThreads, 0, s>>>(B, slots);
    clear_keys_kernel<T, true><<<gk, kThreads, 0, s>>>(G, B);
    rebuild_flip_kernel<<<1, 1, 0, s>>>(B.ctl);
  }

  void launch_strain(cudaStream_t s) {
    if (G.BMAX > 0) strain_kernel<T, true><<<grid_items(cfg.particle_capacity), kThreads, 0, s>>>(G, B);
  }

  unsigned vgrid(int v) const { return (unsigned)(sms * bvariant_minb(v)); }

  // One step as plain launches: strain, the granular tiles, the other tiles
  // (with the step bookkeeping), the rebuild if it was triggered.
  void launch_step(int v, cudaStream_t s) {
    launch_strain(s);
    batch_fn<T>(v, 1)<<<vgrid(v), bvariant_block(v), 0, s>>>(B, 0, 0, 0, cfg.rebuild_every);
    batch_fn<T>(v, 2)<<<vgrid(v), bvariant_block(v), 0, s>>>(B, 0, 0, 0, cfg.rebuild_every);
    launch_rebuild(s);
  }

  int add_step_and_rebuild(cudaGraph_t g, cudaGraphConditionalHandle h, cudaGraphConditionalHandle hl) {
    int cond_bits = 3, every = cfg.rebuild_every;
    void* args[] = {&B, &h, &hl, &cond_bits, &every};
    const cudaGraphNode_t* dep = nullptr;
    size_t ndep = 0;
    cudaGraphNode_t snode;
    if (G.BMAX > 0) {
      void* sargs[] = {&G, &B};
      cudaKernelNodeParams sk = {};
      sk.func = reinterpret_cast<void*>(&strain_kernel<T, true>);
      sk.gridDim = dim3(grid_items(cfg.particle_capacity));
      sk.blockDim = dim3(kThreads);
      sk.kernelParams = sargs;
      TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&snode, g, dep, ndep, &sk));
      dep = &snode;
      ndep = 1;
    }
    cudaKernelNodeParams kp = {};
    kp.func = reinterpret_cast<void*>(batch_fn<T>(variant, 1));
    kp.gridDim = dim3(vgrid(variant));
    kp.blockDim = dim3((unsigned)bvariant_block(variant));
    kp.kernelParams = args;
    cudaGraphNode_t pnode;
    TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&pnode, g, dep, ndep, &kp));
    kp.func = reinterpret_cast<void*>(batch_fn<T>(variant, 2));
    cudaGraphNode_t knode;
    TDEM_CUDA_TRY(&err, cudaGraphAddKernelNode(&knode, g, &pnode, 1, &kp));
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

  // set target -> WHILE { [strain] -> granular tiles -> other tiles -> IF rebuild { ... } }
  int build_graph() {
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
    int rc = add_step_and_rebuild(body, h_reb, h_loop);
    if (rc) return rc;
    TDEM_CUDA_TRY(&err, cudaGraphInstantiate(&exec, graph, 0));
    exec_target = 1;
    return TDEM_OK;
  }

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

  int ensure_stage(size_t m) {
    if (m <= stage_cap) return TDEM_OK;
    if (stage_dev) cudaFree(stage_dev);
    if (bpart_dev) cudaFree(bpart_dev);
    if (bstr_dev) cudaFree(bstr_dev);
    if (stage_host) cudaFreeHost(stage_host);
    if (bpart_host) cudaFreeHost(bpart_host);
    if (bstr_host) cudaFreeHost(bstr_host);
    stage_dev = nullptr;
    bpart_dev = nullptr;
    bstr_dev = nullptr;
    stage_host = nullptr;
    bpart_host = nullptr;
    bstr_host = nullptr;
    stage_cap = 0;
    const size_t bm = (size_t)std::max(G.BMAX, 1);
    TDEM_CUDA_TRY(&err, cudaMalloc(&stage_dev, 9 * m * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&stage_host, 9 * m * sizeof(double)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&bpart_dev, bm * m * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&bpart_host, bm * m * sizeof(int)));
    TDEM_CUDA_TRY(&err, cudaMalloc(&bstr_dev, bm * m * sizeof(float)));
    TDEM_CUDA_TRY(&err, cudaMallocHost(&bstr_host, bm * m * sizeof(float)));
    stage_cap = m;
    return TDEM_OK;
  }

  // First-fit key range; updates key_hi.
  int alloc_keys(int len) {
    for (auto it = free_keys.begin(); it != free_keys.end(); ++it) {
      if (it->second < len) continue;
      const int start = it->first, rest = it->second - len;
      free_keys.erase(it);
      if (rest > 0) free_keys[start + len] = rest;
      used_keys[start] = len;
      key_hi = std::max(key_hi, start + len);
      return start;
    }
    return -1;
  }

  void free_key_range(int start, int len) {
    used_keys.erase(start);
    auto it = free_keys.emplace(start, len).first;
    auto nx = std::next(it);
    if (nx != free_keys.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_keys.erase(nx);
    }
    if (it != free_keys.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_keys.erase(it);
      }
    }
    key_hi = used_keys.empty() ? 0 : std::prev(used_keys.end())->first + std::prev(used_keys.end())->second;
  }

  int admit(const tdem_hm_config& c, const double* pos, const double* vel, const double* omega, const double* radius,
            const double* mass, const double* inertia, const int* bonds, const double* strength, long long nb,
            int* id, cudaStream_t s) override {
    if (!pos || !vel || !omega || !radius || !mass || !inertia || !id)
      return tdem::fail(&err, TDEM_ERR_BADARG, "admit: null state pointer");
    if (c.n < 1) return tdem::fail(&err, TDEM_ERR_BADARG, "admit: n must be >= 1");
    if (c.ncx < 1 || c.ncy < 1 || c.ncx > 65535 || c.ncy > 32767)
      return tdem::fail(&err, TDEM_ERR_BADARG, "admit: cell grid must be 1..65535 x 1..32767");
    if (!(c.cell > 0.0) || !(c.dt > 0.0) || !(c.skin > 0.0) || !(c.young > 0.0))
      return tdem::fail(&err, TDEM_ERR_BADARG, "admit: cell, dt, skin and young must be positive");
    if (!(c.restitution > 0.0 && c.restitution <= 1.0))
      return tdem::fail(&err, TDEM_ERR_BADARG, "admit: restitution must be in (0, 1]");
    if (!(c.inertia_factor > 0.0)) return tdem::fail(&err, TDEM_ERR_BADARG, "admit: inertia_factor must be positive");
    if (nb > 0 && (G.BMAX == 0 || !bonds || !strength))
      return tdem::fail(&err, TDEM_ERR_BADARG, "admit: bonds need a batch with max_bonds > 0 and bond arrays");
    const long long ncells = (long long)c.ncx * c.ncy;
    if (free_slots.empty()) return tdem::fail(&err, TDEM_ERR_CAPACITY, "admit: no free instance slot");
    if (occupied + c.n > cfg.particle_capacity)
      return tdem::fail(&err, TDEM_ERR_CAPACITY, "admit: particle capacity exhausted");
    const int key_off = ncells < (1ll << 31) ? alloc_keys((int)ncells) : -1;
    if (key_off < 0) return tdem::fail(&err, TDEM_ERR_CAPACITY, "admit: no free cell-key range for the grid");
    const int m = c.n;
    auto undo_keys = [&]() { free_key_range(key_off, (int)ncells); };
    // bond slot lists (instance-local ids), bond order per disc
    std::vector<int> part, fill;
    std::vector<float> str;
    if (G.BMAX > 0) {
      part.assign((size_t)G.BMAX * m, -1);
      str.assign((size_t)G.BMAX * m, 1.0f);
      fill.assign((size_t)m, 0);
      for (long long b = 0; b < nb; ++b) {
        const int a = bonds[2 * b], q = bonds[2 * b + 1];
        if (a < 0 || q < 0 || a >= m || q >= m || a == q) {
          undo_keys();
          return tdem::fail(&err, TDEM_ERR_BADARG, "admit: bond " + std::to_string(b) + " has an invalid disc index");
        }
        if (!(strength[b] > 0.0)) {
          undo_keys();
          return tdem::fail(&err, TDEM_ERR_BADARG, "admit: bond strength factors must be positive");
        }
        for (int e : {a, q}) {
          if (fill[e] >= G.BMAX) {
            undo_keys();
            return tdem::fail(&err, TDEM_ERR_BADARG,
                              "admit: disc " + std::to_string(e) + " has more than max_bonds bonds");
          }
          part[(size_t)fill[e] * m + e] = (e == a) ? q : a;
          str[(size_t)fill[e] * m + e] = (float)strength[b];
          ++fill[e];
        }
      }
    }
    int rc = ensure_stage((size_t)m);
    if (rc) {
      undo_keys();
      return rc;
    }
    const int slot = free_slots.back();
    free_slots.pop_back();
    Inst& I = inst[(size_t)slot];
    I = Inst{};
    I.state = 1;
    I.n = m;
    I.key_off = key_off;
    I.nkeys = (int)ncells;
    I.eval0 = evals;
    tdem_hm_config cc = c;
    cc.max_bonds = G.BMAX;
    make_params<T>(cc, G.W, I.par);
    I.par.n = G.n;
    I.par.W = G.W;
    I.par.BMAX = G.BMAX;
    I.par.nkeys = (int)ncells;
    I.par.tiles_x = 0;
    I.par.load_cap = 0;
    I.par.key_off = key_off;
    I.par.eval0 = evals;
    I.par.stop = LLONG_MAX;
    I.par.feat = (nb > 0 || c.indenter_radius > 0.0) ? 1 : 0;
    I.par.prem = G.prem;  // the batch's arrays decide, not the instance's config
    // stage and append
    double* h = stage_host;
    std::memcpy(h, pos, 2 * (size_t)m * sizeof(double));
    std::memcpy(h + 2 * (size_t)m, vel, 2 * (size_t)m * sizeof(double));
    std::memcpy(h + 4 * (size_t)m, omega, (size_t)m * sizeof(double));
    std::memcpy(h + 5 * (size_t)m, radius, (size_t)m * sizeof(double));
    std::memcpy(h + 6 * (size_t)m, mass, (size_t)m * sizeof(double));
    std::memcpy(h + 7 * (size_t)m, inertia, (size_t)m * sizeof(double));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(stage_dev, h, 8 * (size_t)m * sizeof(double), cudaMemcpyHostToDevice, s));
    const double* d = stage_dev;
    const unsigned g = grid_items(m);
    batch_set_params_kernel<T><<<1, 1, 0, s>>>(iparams + slot, I.par);
    batch_append_kernel<T><<<g, kThreads, 0, s>>>(I.par, B, slot, m, d, d + 2 * (size_t)m, d + 4 * (size_t)m,
                                                  d + 5 * (size_t)m, d + 6 * (size_t)m, d + 7 * (size_t)m);
    if (G.BMAX > 0) {
      std::memcpy(bpart_host, part.data(), part.size() * sizeof(int));
      std::memcpy(bstr_host, str.data(), str.size() * sizeof(float));
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(bpart_dev, bpart_host, part.size() * sizeof(int), cudaMemcpyHostToDevice, s));
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(bstr_dev, bstr_host, str.size() * sizeof(float), cudaMemcpyHostToDevice, s));
      batch_bond_init_kernel<T><<<g, kThreads, 0, s>>>(I.par, B, m, bpart_dev, bstr_dev);
    }
    batch_admit_kernel<<<1, 1, 0, s>>>(B.ctl, B.istate, B.iticket, B.iled, slot, m, key_hi);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    // the pinned staging is reused by the next admission: wait for the copies
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    occupied += m;
    live += m;
    need_rebuild = true;
    *id = slot;
    return TDEM_OK;
  }

  // The rebuild that sorts admitted particles in and drops retired ones.
  int settle(cudaStream_t s) {
    if (!need_rebuild) return TDEM_OK;
    request_rebuild_kernel<<<1, 1, 0, s>>>(B.ctl);
    launch_rebuild(s);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    need_rebuild = false;
    occupied = live;
    for (int k : pending_slots) {
      inst[(size_t)k].state = 0;
      free_slots.push_back(k);
    }
    pending_slots.clear();
    for (auto& r : pending_keys) free_key_range(r.first, r.second);
    pending_keys.clear();
    batch_key_hi_kernel<<<1, 1, 0, s>>>(B.ctl, key_hi);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int step(long long n, cudaStream_t s) override {
    int rc = settle(s);  // n == 0 settles admissions and retirements and builds the step graph
    if (rc || n < 0) return rc;
    if (graph_on && !graph_failed && !exec) {
      if (build_graph() != TDEM_OK) {
        graph_failed = true;  // plain launches: the same kernels and results
        destroy_graphs();
        cudaGetLastError();
      }
    }
    if (n == 0) return TDEM_OK;
    if (graph_on && exec) {
      rc = set_graph_target(n);
      if (rc) return rc;
      TDEM_CUDA_TRY(&err, cudaGraphLaunch(exec, s));
    } else {
      for (long long k = 0; k < n; ++k) {
        launch_step(variant, s);
      }
      TDEM_CUDA_TRY(&err, cudaGetLastError());
    }
    evals += n;
    return TDEM_OK;
  }

  int check_id(int id) {
    if (id < 0 || id >= slots || inst[(size_t)id].state != 1)
      return tdem::fail(&err, TDEM_ERR_BADARG, "no live instance with id " + std::to_string(id));
    return TDEM_OK;
  }

  // Read-back evaluation of one instance (no state change).
  int peek(int id, cudaStream_t s) {
    int rc = settle(s);
    if (rc) return rc;
    launch_strain(s);
    batch_state_kernel<<<1, 1, 0, s>>>(B.istate, id, kInstPeek, 0);
    batch_fn<T>(0, 0)<<<(unsigned)(sms * 2), 256, 0, s>>>(B, 0, 0, 0, 0);
    batch_state_kernel<<<1, 1, 0, s>>>(B.istate, id, 0, kInstPeek);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int read(int id, double* pos, double* vel, double* omega, double* force, double* torque, double* ledger, int count,
           cudaStream_t s) override {
    int rc = check_id(id);
    if (rc) return rc;
    if ((rc = peek(id, s))) return rc;
    const Inst& I = inst[(size_t)id];
    const size_t m = (size_t)I.n;
    const bool want_state = pos || vel || omega || force || torque;
    if (want_state) {
      if ((rc = ensure_stage(m))) return rc;
      TDEM_CUDA_TRY(&err, cudaMemsetAsync(stage_dev, 0, 8 * m * sizeof(double), s));
      batch_unpack_kernel<T><<<grid_items((long long)m), kThreads, 0, s>>>(I.par, B, id, (int)m, stage_dev);
      TDEM_CUDA_TRY(&err, cudaGetLastError());
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(stage_host, stage_dev, 8 * m * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_led, B.iled + (size_t)id * kInstLedger, kInstLedger * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_state, B.istate + id, sizeof(int), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    if (want_state) {
      if (pos) std::memcpy(pos, stage_host, 2 * m * sizeof(double));
      if (vel) std::memcpy(vel, stage_host + 2 * m, 2 * m * sizeof(double));
      if (omega) std::memcpy(omega, stage_host + 4 * m, m * sizeof(double));
      if (force) std::memcpy(force, stage_host + 5 * m, 2 * m * sizeof(double));
      if (torque) std::memcpy(torque, stage_host + 7 * m, m * sizeof(double));
    }
    if (ledger && count > 0) assemble_ledger(inst[(size_t)id], host_led, *host_state, ledger, count);
    return TDEM_OK;
  }

  // Per-instance ledger in TDEM_HM_L_* / TDEM_BATCH_L_* order from its device row.
  void assemble_ledger(const Inst& I, const double* L, int st, double* ledger, int count) const {
    const bool primed = evals > I.eval0;
    double v[TDEM_BATCH_L_COUNT] = {0};
    v[TDEM_HM_L_KINETIC] = L[9];
    v[TDEM_HM_L_POTENTIAL] = L[10];
    v[TDEM_HM_L_HERTZ] = L[11];
    v[TDEM_HM_L_TANGENTIAL] = L[12];
    v[TDEM_HM_L_DISSIPATED] = L[0] + L[13];
    v[TDEM_HM_L_BOND_ELASTIC] = L[14];
    v[TDEM_HM_L_FRACTURE] = L[1] + L[15];
    v[TDEM_HM_L_TOOL_WORK] = L[2] + (primed ? L[16] : 0.0);
    v[TDEM_HM_L_BROKEN] = L[3] + L[17];
    v[TDEM_HM_L_TOTAL] = v[TDEM_HM_L_KINETIC] + v[TDEM_HM_L_POTENTIAL] + v[TDEM_HM_L_HERTZ] +
                         v[TDEM_HM_L_TANGENTIAL] + v[TDEM_HM_L_DISSIPATED] + v[TDEM_HM_L_BOND_ELASTIC] +
                         v[TDEM_HM_L_FRACTURE] - v[TDEM_HM_L_TOOL_WORK];
    v[TDEM_HM_L_EVALS] = (double)std::min(evals - I.eval0, I.par.stop);  // a frozen instance stops counting
    v[TDEM_HM_L_REBUILDS] = (double)host_ctl->rebuilds;
    v[TDEM_HM_L_MAX_NEIGHBORS] = (double)host_ctl->max_cnt;
    v[TDEM_HM_L_STATUS] = (double)((st | (st >> kInstRebuildShift)) & 0xFF);
    v[TDEM_HM_L_GRAPH] = exec ? 1.0 : 0.0;
    v[TDEM_HM_L_VARIANT] = (double)variant;
    v[TDEM_BATCH_L_PEAK_LOAD] = L[6];
    v[TDEM_BATCH_L_PEAK_EVAL] = L[7];
    v[TDEM_BATCH_L_REACTION_X] = L[4];
    v[TDEM_BATCH_L_REACTION_Y] = L[5];
    std::memcpy(ledger, v, (size_t)std::min(count, (int)TDEM_BATCH_L_COUNT) * sizeof(double));
  }

  // Ledgers of many instances from one read-back evaluation of all of them.
  int read_ledgers(const int* ids, int count, double* out, cudaStream_t s) override {
    if (count <= 0) return TDEM_OK;
    for (int j = 0; j < count; ++j) {
      int rc = check_id(ids[j]);
      if (rc) return rc;
    }
    int rc = settle(s);
    if (rc) return rc;
    if ((size_t)count > list_cap) {
      if (list_dev) cudaFree(list_dev);
      if (list_host) cudaFreeHost(list_host);
      list_dev = nullptr;
      list_host = nullptr;
      list_cap = 0;
      TDEM_CUDA_TRY(&err, cudaMalloc(&list_dev, (size_t)count * sizeof(int)));
      TDEM_CUDA_TRY(&err, cudaMallocHost(&list_host, (size_t)count * sizeof(int)));
      list_cap = (size_t)count;
    }
    if (all_led.size() < (size_t)slots * kInstLedger) {
      if (all_led_host) cudaFreeHost(all_led_host);
      if (all_state_host) cudaFreeHost(all_state_host);
      all_led_host = nullptr;
      all_state_host = nullptr;
      TDEM_CUDA_TRY(&err, cudaMallocHost(&all_led_host, (size_t)slots * kInstLedger * sizeof(double)));
      TDEM_CUDA_TRY(&err, cudaMallocHost(&all_state_host, (size_t)slots * sizeof(int)));
      all_led.resize((size_t)slots * kInstLedger);
    }
    std::memcpy(list_host, ids, (size_t)count * sizeof(int));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(list_dev, list_host, (size_t)count * sizeof(int), cudaMemcpyHostToDevice, s));
    launch_strain(s);
    const unsigned g = grid_items(count);
    batch_state_list_kernel<<<g, kThreads, 0, s>>>(B.istate, list_dev, count, kInstPeek, 0);
    batch_fn<T>(0, 0)<<<(unsigned)(sms * 2), 256, 0, s>>>(B, 0, 0, 0, 0);
    batch_state_list_kernel<<<g, kThreads, 0, s>>>(B.istate, list_dev, count, 0, kInstPeek);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(all_led_host, B.iled, (size_t)slots * kInstLedger * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(all_state_host, B.istate, (size_t)slots * sizeof(int),
                                        cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    for (int j = 0; j < count; ++j)
      assemble_ledger(inst[(size_t)ids[j]], all_led_host + (size_t)ids[j] * kInstLedger, all_state_host[ids[j]],
                      out + (size_t)j * TDEM_BATCH_L_COUNT, TDEM_BATCH_L_COUNT);
    return TDEM_OK;
  }

  int set_steps(int id, long long steps, cudaStream_t s) override {
    int rc = check_id(id);
    if (rc) return rc;
    if (steps < 0) return tdem::fail(&err, TDEM_ERR_BADARG, "set_steps: steps must be >= 0");
    Inst& I = inst[(size_t)id];
    I.par.stop = steps == 0 ? LLONG_MAX : steps;
    batch_set_params_kernel<T><<<1, 1, 0, s>>>(iparams + id, I.par);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int retire(int id, cudaStream_t s) override {
    int rc = check_id(id);
    if (rc) return rc;
    batch_state_kernel<<<1, 1, 0, s>>>(B.istate, id, 0, kInstAlive | kInstPeek);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    Inst& I = inst[(size_t)id];
    I.state = 2;
    live -= I.n;
    pending_slots.push_back(id);
    pending_keys.emplace_back(I.key_off, I.nkeys);
    need_rebuild = true;
    return TDEM_OK;
  }

  int read_bonds(int id, int* pairs, int* state, long long cap, long long* count, cudaStream_t s) override {
    int rc = check_id(id);
    if (rc) return rc;
    if ((rc = settle(s))) return rc;
    if (G.BMAX == 0) {
      if (count) *count = 0;
      return TDEM_OK;
    }
    const Inst& I = inst[(size_t)id];
    const long long want = std::max(cap, 0ll);
    int* dp = nullptr;
    int* ds = nullptr;
    if (want > 0) {
      TDEM_CUDA_TRY(&err, cudaMallocAsync(&dp, 2 * want * sizeof(int), s));
      TDEM_CUDA_TRY(&err, cudaMallocAsync(&ds, 2 * want * sizeof(int), s));
    }
    TDEM_CUDA_TRY(&err, cudaMemsetAsync(count_dev, 0, sizeof(unsigned long long), s));
    batch_bonds_out_kernel<T><<<grid_items(I.n), kThreads, 0, s>>>(I.par, B, id, dp, ds, want, count_dev);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(count_host, count_dev, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    const long long got = (long long)*count_host;
    const long long copy = std::min(got, want);
    if (copy > 0) {
      TDEM_CUDA_TRY(&err, cudaMemcpy(pairs, dp, 2 * copy * sizeof(int), cudaMemcpyDeviceToHost));
      TDEM_CUDA_TRY(&err, cudaMemcpy(state, ds, 2 * copy * sizeof(int), cudaMemcpyDeviceToHost));
    }
    if (dp) cudaFreeAsync(dp, s);
    if (ds) cudaFreeAsync(ds, s);
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    if (count) *count = got;
    return got > want ? tdem::fail(&err, TDEM_ERR_CAPACITY, "bond output capacity too small") : TDEM_OK;
  }

  int info(long long* out, int count, cudaStream_t s) override {
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    long long v[TDEM_BATCH_I_COUNT] = {0};
    v[TDEM_BATCH_I_LIVE_PARTICLES] = host_ctl->n_live;
    long long ninst = 0;
    for (const Inst& I : inst) ninst += (I.state == 1);
    v[TDEM_BATCH_I_LIVE_INSTANCES] = ninst;
    v[TDEM_BATCH_I_EVALS] = host_ctl->evals;
    v[TDEM_BATCH_I_REBUILDS] = host_ctl->rebuilds;
    v[TDEM_BATCH_I_TILES] = host_ctl->ntiles;
    v[TDEM_BATCH_I_PARTICLE_CAPACITY] = cfg.particle_capacity;
    v[TDEM_BATCH_I_BYTES] = (long long)arena.size;
    v[TDEM_BATCH_I_KEY_HI] = host_ctl->key_hi;
    v[TDEM_BATCH_I_STATUS] = host_ctl->status;
    v[TDEM_BATCH_I_VARIANT] = variant;
    v[TDEM_BATCH_I_GRAPH] = exec ? 1 : 0;
    v[TDEM_BATCH_I_MAX_NEIGHBORS] = host_ctl->max_cnt;
    std::memcpy(out, v, (size_t)std::min(count, (int)TDEM_BATCH_I_COUNT) * sizeof(long long));
    return TDEM_OK;
  }

  int set_variant(int v) override {
    if (v < 0 || v >= kBatchVariants) return tdem::fail(&err, TDEM_ERR_BADARG, "variant out of range");
    if (v != variant) {
      variant = v;
      destroy_graphs();
    }
    return TDEM_OK;
  }
  int get_variant() const override { return variant; }

  // Time `steps` real steps of each variant (they advance every instance)
  // and keep the fastest. Plain launches, rebuilds included.
  int autotune(int steps, cudaStream_t s, float* ms_out) override {
    if (steps < 1) return tdem::fail(&err, TDEM_ERR_BADARG, "autotune needs steps >= 1");
    int rc = settle(s);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    TDEM_CUDA_TRY(&err, cudaEventCreate(&e0));
    TDEM_CUDA_TRY(&err, cudaEventCreate(&e1));
    int best = variant;
    float best_ms = 1e30f;
    for (int v = 0; v < kBatchVariants; ++v) {
      TDEM_CUDA_TRY(&err, cudaEventRecord(e0, s));
      for (int k = 0; k < steps; ++k) {
        launch_step(v, s);
      }
      TDEM_CUDA_TRY(&err, cudaEventRecord(e1, s));
      TDEM_CUDA_TRY(&err, cudaEventSynchronize(e1));
      float ms = 0.0f;
      TDEM_CUDA_TRY(&err, cudaEventElapsedTime(&ms, e0, e1));
      if (ms_out) ms_out[v] = ms;
      evals += steps;
      if (ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return set_variant(best);
  }

  int use_graph(int on) override {
    graph_on = on != 0;
    return TDEM_OK;
  }
};

}  // namespace

struct tdem_batch {
  std::unique_ptr<BatchBase> e;
};

namespace {
std::string g_batch_create_error;
}

extern "C" {

int tdem_batch_create(const tdem_batch_config* c, tdem_batch** out) {
  if (!c || !out) return tdem::fail(&g_batch_create_error, TDEM_ERR_BADARG, "null argument");
  *out = nullptr;
  int rc = Batch<float>::check_config(*c, g_batch_create_error);
  if (rc) return rc;
  auto h = std::make_unique<tdem_batch>();
  if (c->precision == 64) {
    auto e = std::make_unique<Batch<double>>();
    rc = e->init(*c);
    if (rc) {
      g_batch_create_error = e->err;
      return rc;
    }
    h->e = std::move(e);
  } else {
    auto e = std::make_unique<Batch<float>>();
    rc = e->init(*c);
    if (rc) {
      g_batch_create_error = e->err;
      return rc;
    }
    h->e = std::move(e);
  }
  *out = h.release();
  return TDEM_OK;
}

void tdem_batch_destroy(tdem_batch* h) { delete h; }

int tdem_batch_admit(tdem_batch* h, const tdem_hm_config* inst, const double* pos, const double* vel,
                     const double* omega, const double* radius, const double* mass, const double* inertia,
                     const int32_t* bond_pairs, const double* bond_strength, int64_t n_bonds, int32_t* out_id,
                     void* stream) {
  if (!h || !inst) return TDEM_ERR_BADARG;
  int id = -1;
  const int rc = h->e->admit(*inst, pos, vel, omega, radius, mass, inertia, bond_pairs, bond_strength,
                             (long long)n_bonds, &id, static_cast<cudaStream_t>(stream));
  if (out_id) *out_id = id;
  return rc;
}

int tdem_batch_step(tdem_batch* h, int64_t n_steps, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->step((long long)n_steps, static_cast<cudaStream_t>(stream));
}

int tdem_batch_read(tdem_batch* h, int32_t id, double* pos, double* vel, double* omega, double* force,
                    double* torque, double* ledger, int32_t ledger_count, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->read(id, pos, vel, omega, force, torque, ledger, ledger_count, static_cast<cudaStream_t>(stream));
}

int tdem_batch_read_ledgers(tdem_batch* h, const int32_t* ids, int32_t count, double* out, void* stream) {
  if (!h || (count > 0 && (!ids || !out))) return TDEM_ERR_BADARG;
  return h->e->read_ledgers(ids, count, out, static_cast<cudaStream_t>(stream));
}

int tdem_batch_set_steps(tdem_batch* h, int32_t id, int64_t steps, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->set_steps(id, (long long)steps, static_cast<cudaStream_t>(stream));
}

int tdem_batch_retire(tdem_batch* h, int32_t id, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->retire(id, static_cast<cudaStream_t>(stream));
}

int tdem_batch_read_bonds(tdem_batch* h, int32_t id, int32_t* pairs, int32_t* state, int64_t capacity,
                          int64_t* count, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->read_bonds(id, pairs, state, (long long)capacity, &c, static_cast<cudaStream_t>(stream));
  if (count) *count = (int64_t)c;
  return rc;
}

int tdem_batch_info(tdem_batch* h, int64_t* out, int32_t count, void* stream) {
  if (!h || !out) return TDEM_ERR_BADARG;
  long long v[TDEM_BATCH_I_COUNT];
  const int rc = h->e->info(v, TDEM_BATCH_I_COUNT, static_cast<cudaStream_t>(stream));
  for (int k = 0; k < std::min<int>(count, TDEM_BATCH_I_COUNT); ++k) out[k] = (int64_t)v[k];
  return rc;
}

int tdem_batch_bytes(const tdem_batch_config* c, int64_t* bytes) {
  if (!c || !bytes) return TDEM_ERR_BADARG;
  std::string e;
  int rc = Batch<float>::check_config(*c, e);
  if (rc) return rc;
  if (c->precision == 64) {
    Batch<double> b;
    b.cfg = *c;
    b.slots = c->max_instances;
    b.G.W = c->max_neighbors;
    b.G.BMAX = c->max_bonds;
    Arena a;
    b.carve(a);
    *bytes = (int64_t)(a.used + 256);
  } else {
    Batch<float> b;
    b.cfg = *c;
    b.slots = c->max_instances;
    b.G.W = c->max_neighbors;
    b.G.BMAX = c->max_bonds;
    Arena a;
    b.carve(a);
    *bytes = (int64_t)(a.used + 256);
  }
  return TDEM_OK;
}

int tdem_batch_num_variants(void) { return kBatchVariants; }

int tdem_batch_set_variant(tdem_batch* h, int variant) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->set_variant(variant);
}

int tdem_batch_get_variant(const tdem_batch* h) { return h ? h->e->get_variant() : -1; }

int tdem_batch_autotune(tdem_batch* h, int steps, float* ms_out, void* stream) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->autotune(steps, static_cast<cudaStream_t>(stream), ms_out);
}

int tdem_batch_use_graph(tdem_batch* h, int on) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->use_graph(on);
}

int tdem_batch_last_error(const tdem_batch* h, char* buf, size_t len) {
  if (!buf || len == 0) return TDEM_ERR_BADARG;
  const std::string& m = h ? h->e->err : g_batch_create_error;
  const size_t k = std::min(len - 1, m.size());
  std::memcpy(buf, m.data(), k);
  buf[k] = '\0';
  return TDEM_OK;
}

}  // extern "C"
