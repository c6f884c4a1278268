// Device-side data model of the Hertz-Mindlin 2-D disc engine.
//
// HBM layout (all per-particle arrays in the current sorted order; sorted by
// a tiled Morton key of the cell so that neighbours in space are neighbours
// in memory):
//   pos[2][N]   V4 (x offset, y offset, radius, cell)     ping-pong per step
//               cell = cx | cy << 16, the particle's integer cell origin,
//               bit-cast into the last lane (exact in both precisions)
//   vel[2][N]   V4 (vx, vy, omega, 1/m)                   ping-pong per step
//   head[2][N]  uint4 {word, partner of slot 0, slot 1, slot 2}: one 16-byte
//               load gives the count, the history mask and the first three
//               partners, so all their position gathers issue together;
//               word = candidate count (bits 0..7) | mask of slots whose
//               stored tangential history is non-zero (bits 8..31)
//   nbr[2][(W-3)*N] uint32 slot-major partners of slots 3 .. W-1
//   hist[2][W*N] V2 tangential history of (particle, slot partner), one copy
//               per side, both in the orientation of the pair's lower sorted
//               index; both partners update their copy in place with the same
//               arithmetic on the same operands, so the copies stay identical
//   orig[2][N]  int original particle id
//   whist[2][4N] V2 wall tangential history (4 walls)
//   bond slots (bonded sheets only), slot-major [BMAX*N], swapped at a rebuild:
//   bpart       uint32 partner sorted index (bits 0..28), failure mode
//               (bits 29..30: 1 tensile, 2 shear, 3 both) and broken (bit 31)
//   bref        V2 reference bond vector x0(partner) - x0(self)
//   bstr        T  strength factor of the bond (scales both break strains)
//   bus         V2 shear displacement of the bond, in the orientation of the
//               pair's lower sorted index (one copy per side, kept identical)
//   bfail       int evaluation index at which the bond broke (-1: intact)
//   bcnt[N]     int initial bonds of the disc; bpinv[N] V4 constant
//               pseudo-inverse of the disc's bond covariance (row major)
// head / nbr / hist / orig / whist / bond slots swap at a rebuild. Position =
// (cx * cell + x offset, cy * cell + y offset): FP32 offsets from an integer
// cell origin keep contact geometry exact to ~ulp(cell) anywhere in a large
// box. The moment of inertia is kappa m r^2 with one kappa per engine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace tdem {
namespace hm {

constexpr int kMaxSlots = 24;
constexpr int kThreads = 256;

enum Status : int {
  kStatusCapacity = 1,   // a particle had more candidates than slots
  kStatusNonfinite = 2,  // non-finite position or velocity
  kStatusEscaped = 4,    // a particle left the cell grid by more than a cell
  kStatusInertia = 8,    // an uploaded moment of inertia was not kappa m r^2
  kStatusTimeout = 16,   // a bounded wait on a bulk copy ran out
};

template <class T>
struct alignas(4 * sizeof(T)) V4 {
  T x, y, z, w;
};
template <class T>
struct alignas(2 * sizeof(T)) V2 {
  T x, y;
};

template <class T>
struct Params {
  int n;          // particles
  int W;          // slots per particle (ELL width)
  int ncx, ncy;   // cell grid; walls sit at 0, ncx*cell and 0, ncy*cell
  int tiles_x;    // 32x32-cell tiles along x (key = tile-major, Morton inside a tile)
  int nkeys;      // size of the key space
  int walls;      // bit 0 left, 1 right, 2 bottom, 3 top
  T cell, inv_cell, skin, dt, half_dt;
  T estar2;       // 2 E*
  T gstar8;       // 8 G*
  T damp;         // 2 sqrt(5/6) beta (Tsuji)
  T mu, mu_wall;
  T gx, gy;       // gravity (acceleration)
  T kinv;         // 1 / kappa, with I = kappa m r^2
  float rebuild_disp;  // rebuild once the displacement bound exceeds this
  // bonded-particle model (BMAX == 0: no bonds)
  int BMAX;
  T kn, ks;       // bond normal and shear stiffness (N/m)
  T bzeta;        // bond damping ratio: c = 2 zeta sqrt(k m*)
  T cn_k, cs_k;   // 2 zeta sqrt(kn), 2 zeta sqrt(ks): c = c_k / sqrt(1/m_a + 1/m_b)
  double eps_t, eps_s;  // tensile and objective-shear break strains
  // rigid circular indenter (irad == 0: none), Hertz normal + dashpot
  double ind_x0, ind_y0, ind_vx, ind_vy;
  T irad;
  int load_cap;   // capacity of the per-evaluation indenter load record
  int ind_slots;  // indenter partials: entries of the first half of Bufs::ind_part (the second half: sorted)
  // batched engine: one Params per instance (n = the particle capacity, the
  // stride of every slot-major array)
  int key_off;       // first cell key of the instance (key = key_off + cy * ncx + cx)
  long long eval0;   // batch evaluation index of the instance's first step
  long long stop;    // the instance's own step limit: frozen once it has taken `stop` steps
  int feat;          // 1: the instance has bonds or an indenter (stepped by the bonded kernel build)
  int prem;          // FP32: positions carry their rounding remainder (Bufs::prem)
  // FP32 screens that keep FP64 off the common path (decisions unchanged):
  // float brackets of the break strains (largest float <= eps, smallest >= eps)
  float eps_t_lo, eps_t_hi, eps_s_lo, eps_s_hi;
  // indenter centre at evaluation 0 and its displacement per evaluation
  float ind_x0f, ind_y0f, ind_dxf, ind_dyf;
  // SM clock cycles a bounded wait of the bulk-copy kernels may take (about
  // a second by default; tests of the failure path shorten it)
  long long wait_budget;
};

constexpr unsigned kBondIdx = (1u << 29) - 1u;
constexpr unsigned kBondBroken = 1u << 31;
constexpr int kBondModeShift = 29;
constexpr int kMaxBondSlots = 8;

// Device control block: buffer parities, the rebuild trigger and status.
struct Ctl {
  int sp;                  // current pos/vel/hist buffer
  int lp;                  // current list / cell / orig / wall-history buffer
  unsigned ticket;         // completed blocks of the running step kernel
  int rebuild_pending;     // a rebuild must run before the next evaluation
  // max |v|^2 of the running step (float bits) and the Status bits: one
  // aligned 8-byte pair, so a step's last block reads both in one load
  alignas(8) unsigned vmax2_bits;
  int status;
  float disp;              // displacement bound since the last rebuild
  int rebuilds;
  int max_cnt;             // largest candidate count of the last rebuild
  int tile_next2;          // batched engine: chunk counter of the second step launch
  long long evals;         // force evaluations committed (prime + steps)
  long long target;        // stop the step loop at this many evaluations
  double tool_work;        // work done by the indenter on the discs (J)
  double reaction_x, reaction_y;  // ice-on-indenter force of the last evaluation
  unsigned load_entries;   // entries in the per-evaluation indenter list
  int broken;              // bonds broken so far
  // batched engine
  int n_live;              // particles in the sorted arrays [0, n_live)
  int n_old;               // n_live when the running rebuild started
  int ntiles;              // 32-particle tiles of the live instances
  int ntiles_plain;        // of which the first ones belong to instances without bonds or indenter
  int since;               // steps since the last rebuild
  int key_hi;              // dead-particle key: one past the highest allocated cell key
  int tile_next;           // next tile chunk handed out by the (first) step launch
};

// Batched engine: per-instance state word (low byte: Status bits of the
// instance) and the fixed tile width (one warp per tile).
constexpr int kInstAlive = 1 << 8;   // stepped; cleared when the instance retires
constexpr int kInstPeek = 1 << 9;    // selected for the next read-back evaluation
constexpr int kInstRebuildShift = 16;  // Status bits found by a rebuild (bits 16..23)
constexpr int kTile = 32;
constexpr int kTileVals = 12;        // per-tile ledger partial row
constexpr int kInstLedger = 24;      // per-instance ledger row (doubles)

template <class T>
struct Bufs {
  V4<T>* pos[2];
  V4<T>* vel[2];
  uint4* head[2];
  unsigned* nbr[2];
  V2<T>* hist[2];
  int* orig[2];
  V2<T>* whist[2];
  // rebuild scratch
  int* cell_count;
  int* cell_start;
  int* cell_fill;
  int* perm;
  int* block_sums;
  int* tmp_cell;
  V2<T>* tmp_off;
  // ledger and read-back
  double* diss_part;   // per step-kernel warp: committed dissipation (J)
  double* peek_part;   // per block x 8: kinetic, potential, Hertz, tangential, dissipation
  V4<T>* peek_vel;     // integer-time velocity (vx, vy, omega, -)
  V4<T>* peek_force;   // integer-time force (fx, fy, torque, -)
  Ctl* ctl;
  // bonded-particle model
  unsigned* bpart[2];
  V2<T>* bref[2];
  T* bstr[2];
  V2<T>* bus[2];
  int* bfail[2];
  int* bcnt[2];
  V4<T>* bpinv[2];
  T* strain;           // per-disc objective shear invariant of this evaluation
  int* invperm;        // rebuild: old sorted index -> new
  double* frac_part;   // per step-kernel warp: fracture energy released (J)
  double* peek_bond;   // per block: bond elastic energy (read-back)
  // indenter: per-evaluation partial reactions (warp id, fx, fy) and the load record
  double* ind_part;    // [6 * nwarp_slots]: entries (warp id, fx, fy), then the same in warp order
  double* load;        // [2 * load_cap]: reaction (x, y) per evaluation
  // batched engine (null for a single solve)
  int* inst[2];        // instance slot of each particle, swapped at a rebuild
  const Params<T>* iparams;  // per instance slot
  int* istate;         // per instance slot: kInstAlive | kInstPeek | Status bits
  int4* irange;        // per instance slot: {first sorted index, end, first tile, tiles}
  int4* tiles;         // {instance, first sorted index, count, -} per tile
  double* tpart;       // [tiles * kTileVals] per-tile ledger partials
  unsigned* iticket;   // per instance slot: tiles finished in the running kernel
  double* iled;        // [slots * kInstLedger] per-instance ledger
  int* tmp_key;        // rebuild: cell key of each old particle
  int* ifirst;         // [2 * slots]: first tile of each slot, plain instances then the others
  // FP32 position remainders (Params::prem): the exact position of a disc is
  // its cell origin + FP32 offset + this FP32 pair. Indexed by the list
  // parity lp: a step updates its own disc's pair in place, a rebuild
  // gathers them into the other array in the new order.
  float2* prem[2];
};

// The cell id rides in the last lane of the position vector: bit-cast for
// FP32, an exactly representable integer for FP64.
__device__ __forceinline__ float cell_to_lane(int c, float) { return __int_as_float(c); }
__device__ __forceinline__ double cell_to_lane(int c, double) { return (double)c; }
__device__ __forceinline__ int lane_to_cell(float x) { return __float_as_int(x); }
__device__ __forceinline__ int lane_to_cell(double x) { return (int)x; }

constexpr int kHeadSlots = 3;

// Partner of slot s of particle i.
__device__ __forceinline__ int slot_partner(const uint4& h, const unsigned* tail, size_t n, int i, int s) {
  return s == 0 ? (int)h.y : s == 1 ? (int)h.z : s == 2 ? (int)h.w : (int)tail[(size_t)(s - kHeadSlots) * n + i];
}

// Compensated (float-float) accumulator: the sum of FP32 terms kept to about
// 48 bits, in a fixed order. Plain double for the FP64 engine.
template <class T>
struct Acc;
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double get() const { return s; }
};
template <>
struct Acc<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += err;
  }
  __device__ __forceinline__ float get() const { return hi + lo; }
};

// Plain FP64 sum of the engine's terms (the FP64-sum form of an FP32
// engine): every add in double, rounded to the engine's type once at the end.
template <class T>
struct AccD {
  double s = 0.0;
  __device__ __forceinline__ void add(T x) { s += (double)x; }
  __device__ __forceinline__ T get() const { return (T)s; }
};

// The per-particle accumulator: float-float / double (S64 false), or double
// sums for an FP32 engine (S64 true).
template <class T, bool S64>
struct AccSel {
  using type = Acc<T>;
};
template <class T>
struct AccSel<T, true> {
  using type = AccD<T>;
};

__device__ __forceinline__ unsigned spread5(unsigned v) {
  v &= 31u;
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// Tile-major key, Morton order inside each 32x32-cell tile.
__host__ __device__ __forceinline__ int tile_key(int cx, int cy, int tiles_x) {
#ifdef __CUDA_ARCH__
  const unsigned m = spread5((unsigned)cx) | (spread5((unsigned)cy) << 1);
#else
  unsigned m = 0;
  for (int b = 0; b < 5; ++b) m |= (((unsigned)cx >> b) & 1u) << (2 * b) | (((unsigned)cy >> b) & 1u) << (2 * b + 1);
#endif
  return (((cy >> 5) * tiles_x + (cx >> 5)) << 10) | (int)m;
}

}  // namespace hm
}  // namespace tdem
