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
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "hm2d_dev.cuh"

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
  virtual int fragments(int* labels, long long* count, cudaStream_t s) = 0;
  virtual int step_kernel(cudaStream_t s) = 0;
  virtual int rebuild_pending(cudaStream_t s) = 0;
  virtual int get_variant() const = 0;
  virtual int autotune(int steps, cudaStream_t s, float* ms_out) = 0;
  virtual int rebuild(cudaStream_t s) = 0;
  virtual int read_history(int* pairs, double* xi, long long capacity, long long* count, cudaStream_t s) = 0;
  virtual int set_wait_budget(long long cycles) = 0;
  std::string err;
};

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

// Fragments: connected components of the intact bond graph. Every root
// points to itself; a hook links the larger of two roots under the smaller
// one (parents only ever decrease), so the final root of a component is its
// smallest sorted index. Path halving during finds is a benign race for the
// same reason.
__device__ __forceinline__ int cc_find(int* parent, int x) {
  int p = parent[x];
  while (p != x) {
    const int gp = parent[p];
    if (gp != p) parent[x] = gp;
    x = p;
    p = gp;
  }
  return x;
}

template <class T>
__global__ void cc_init_kernel(Params<T> P, int* parent, int* label) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  parent[i] = i;
  label[i] = INT_MAX;
}

template <class T>
__global__ void cc_hook_kernel(Params<T> P, Bufs<T> B, int* parent, int* changed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const int lp = B.ctl->lp;
  const int bc = B.bcnt[lp][i];
  for (int s = 0; s < bc; ++s) {
    const unsigned w = B.bpart[lp][(size_t)s * P.n + i];
    if (w & kBondBroken) continue;
    const int j = (int)(w & kBondIdx);
    if (j <= i) continue;  // each bond once
    const int ri = cc_find(parent, i), rj = cc_find(parent, j);
    if (ri != rj) {
      atomicMin(&parent[max(ri, rj)], min(ri, rj));
      *changed = 1;
    }
  }
}

template <class T>
__global__ void cc_compress_kernel(Params<T> P, int* parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.n) parent[i] = cc_find(parent, i);
}

// Label of a component: its smallest original id; count the roots.
template <class T>
__global__ void cc_label_kernel(Params<T> P, Bufs<T> B, const int* parent, int* label, unsigned long long* roots) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  atomicMin(&label[parent[i]], B.orig[B.ctl->lp][i]);
  if (parent[i] == i) atomicAdd(roots, 1ull);
}

template <class T>
__global__ void cc_out_kernel(Params<T> P, Bufs<T> B, const int* parent, const int* label, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.n) out[B.orig[B.ctl->lp][i]] = label[parent[i]];
}

// The rebuild pipeline (every kernel a no-op unless ctl->rebuild_pending).
template <class T>
void launch_rebuild_seq(const Params<T>& P, const Bufs<T>& B, cudaStream_t s) {
  const int nb = (P.n + kThreads - 1) / kThreads;
  const int nk = (P.nkeys + kThreads - 1) / kThreads;
  const int sb = (P.nkeys + kScanChunk - 1) / kScanChunk;
  bin_kernel<T><<<nb, kThreads, 0, s>>>(P, B);
  scan_blocks_kernel<<<sb, kScanThreads, 0, s>>>(B.ctl, B.cell_count, B.cell_start, B.block_sums, P.nkeys);
  scan_top_kernel<<<1, kScanThreads, 0, s>>>(B.ctl, B.block_sums, P.nkeys);
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
// block shapes; 4..5 = bulk-copy staging of own state; 6 = neighbour window in
// shared memory; 7..8 = per-thread cp.async pipeline, three discs deep, at 3
// and 4 blocks per SM; 9..10 = the same pipeline with one 1024-thread CTA
// per SM, CTA-major and warp-major chunk order; 11 = the pipeline with one
// 512-thread CTA per SM (128 registers: the bonded build without spills; it
// also stages each disc's bond slot words one disc ahead).
// Variants 6..11 are FP32 kernels; an FP64 engine runs variant 1's kernel
// for them.
constexpr int kVariants = 12;
constexpr int kAsyncHalfVariant = 11;
constexpr int kWindowVariant = 6;
constexpr int kAsyncVariant = 7;       // 7, 8: 256-thread CTAs
constexpr int kAsyncWideVariant = 9;   // 9, 10: one 1024-thread CTA per SM
constexpr int kWideBlock = 1024;

template <class T>
using StepFn = void (*)(Params<T>, Bufs<T>, cudaGraphConditionalHandle, cudaGraphConditionalHandle, int, int,
                        StepHint);

// The neighbour-window kernel for FP32 engines; variant 1's kernel for FP64.
template <class T, int MODE, bool F>
StepFn<T> window_fn() {
  if constexpr (sizeof(T) == 4)
    return &force_kernel_win<T, MODE, F>;
  else
    return &force_kernel_pf<T, MODE, 256, 3, F>;
}

// The cp.async pipeline for FP32 engines; variant 1's kernel for FP64.
template <class T, int MODE, int MINB, bool F, int BLOCK = 256, bool WMAJ = false, bool PW = false>
StepFn<T> async_fn() {
  if constexpr (sizeof(T) == 4)
    return &force_kernel_async<T, MODE, BLOCK, MINB, F, WMAJ, PW>;
  else
    return &force_kernel_pf<T, MODE, 256, 3, F>;
}

// The FP64-sum form of an FP32 engine: every variant runs the grid-stride
// kernel with double per-particle sums.
template <class T, bool F>
StepFn<T> step_fn_sum64(int mode) {
  return mode == kPrime ? &force_kernel_pf<T, kPrime, 256, 3, F, true> : &force_kernel_pf<T, kStep, 256, 3, F, true>;
}

template <class T, int MODE, bool F>
StepFn<T> step_fn_mode(int variant) {
  switch (variant) {
    case 1: return &force_kernel_pf<T, MODE, 256, 3, F>;
    case 2: return &force_kernel_pf<T, MODE, 128, 6, F>;
    case 3: return &force_kernel_pf<T, MODE, 256, 2, F>;
    case 4: return &force_kernel_bulk<T, MODE, 256, 3, F>;
    case 5: return &force_kernel_bulk<T, MODE, 128, 6, F>;
    case kWindowVariant: return window_fn<T, MODE, F>();
    case kAsyncVariant: return async_fn<T, MODE, 3, F>();
    case kAsyncVariant + 1: return async_fn<T, MODE, 4, F>();
    case kAsyncWideVariant: return async_fn<T, MODE, 1, F, kWideBlock>();
    case kAsyncWideVariant + 1: return async_fn<T, MODE, 1, F, kWideBlock, true>();
    case kAsyncHalfVariant: return async_fn<T, MODE, 1, F, kWideBlock / 2, true, F>();
    default: return &force_kernel<T, MODE, F>;
  }
}

template <class T, bool F>
StepFn<T> step_fn_feat(int variant, int mode) {
  return mode == kPrime ? step_fn_mode<T, kPrime, F>(variant) : step_fn_mode<T, kStep, F>(variant);
}

// FEAT kernels carry the bonded-particle model and the indenter; the plain
// granular kernels compile without them (fewer registers).
template <class T>
StepFn<T> step_fn(int variant, int mode, bool feat, bool sum64 = false) {
  if (sum64) return feat ? step_fn_sum64<T, true>(mode) : step_fn_sum64<T, false>(mode);
  return feat ? step_fn_feat<T, true>(variant, mode) : step_fn_feat<T, false>(variant, mode);
}

template <class T>
inline int variant_block(int variant) {
  if (variant == kWindowVariant) return sizeof(T) == 4 ? kWinThreads : 256;
  if (variant == kAsyncHalfVariant) return sizeof(T) == 4 ? kWideBlock / 2 : 256;
  if (variant >= kAsyncWideVariant) return sizeof(T) == 4 ? kWideBlock : 256;
  return (variant == 2 || variant == 5) ? 128 : 256;
}

// Dynamic shared memory of a variant's step kernel.
template <class T>
inline size_t variant_smem(int variant, bool prem) {
  if (sizeof(T) != 4) return 0;
  if (variant == kWindowVariant) return kWinSmem;
  if (variant == kAsyncHalfVariant) return async_smem(kWideBlock / 2, prem);
  if (variant >= kAsyncWideVariant) return async_smem(kWideBlock, prem);
  if (variant >= kAsyncVariant) return async_smem(256, prem);
  return 0;
}

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
  int sgrid = 1;  // grid of the pipelined strain kernel (FP32 engines with bonds)
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
  // The device's buffer parities and evaluation count as last read by the
  // host, kept current across plain step launches and explicit rebuilds;
  // invalid after anything that changes them on the device unseen.
  bool sum64 = false;  // FP32 engine with double per-particle sums
  bool mirror_ok = false;
  int m_sp = 0, m_lp = 0;
  long long m_evals = 0;
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

  // host_ctl was just read from the device with nothing enqueued after it
  void refresh_mirror() {
    m_sp = host_ctl->sp;
    m_lp = host_ctl->lp;
    m_evals = host_ctl->evals;
    mirror_ok = true;
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
    sum64 = sizeof(T) == 4 && c.sum_precision == 64;
    P.prem = (sizeof(T) == 4 && c.position_remainder) ? 1 : 0;
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
      const int bs = block_of(v);
      const size_t smem = smem_of(v);
      if (smem > 0)
        for (int mode : {kPrime, kStep})
          TDEM_CUDA_TRY(&err, cudaFuncSetAttribute(reinterpret_cast<const void*>(step_fn<T>(v, mode, feat(), sum64)),
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      TDEM_CUDA_TRY(&err, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &per_sm, reinterpret_cast<const void*>(step_fn<T>(v, kStep, feat(), sum64)), bs, smem));
      const int need = (int)((n + bs - 1) / bs);
      vgrid[v] = std::max(1, std::min(need, per_sm * sms));
      nwarp_slots = std::max(nwarp_slots, vgrid[v] * (bs / 32));
    }
    P.ind_slots = nwarp_slots;
    if (sizeof(T) == 4 && P.BMAX > 0) {
      // the pipelined strain kernel: resident blocks per SM x SMs
      int per_sm = 0;
      TDEM_CUDA_TRY(&err, cudaFuncSetAttribute(reinterpret_cast<const void*>(&strain_kernel_async<float>),
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStrainSmem));
      TDEM_CUDA_TRY(&err, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &per_sm, reinterpret_cast<const void*>(&strain_kernel_async<float>), kStrainBlock,
                              kStrainSmem));
      sgrid = std::max(1, std::min((int)((n + kStrainBlock - 1) / kStrainBlock), per_sm * sms));
    }
    int rc = TDEM_OK;
    for (int b = 0; b < 2 && !rc; ++b) {
      if ((rc = alloc(&B.pos[b], n)) || (rc = alloc(&B.vel[b], n)) || (rc = alloc(&B.head[b], n)) ||
          (rc = alloc(&B.orig[b], n)) || (rc = alloc(&B.whist[b], 4 * n)) ||
          (rc = alloc(&B.nbr[b], (W > 3 ? W - 3 : 1) * n)) ||
          (rc = alloc(&B.hist[b], W * n)))
        return rc;
      if (P.prem && (rc = alloc(&B.prem[b], n))) return rc;
    }
    if ((rc = alloc(&B.cell_count, (size_t)P.nkeys)) || (rc = alloc(&B.cell_start, (size_t)P.nkeys)) ||
        (rc = alloc(&B.cell_fill, (size_t)P.nkeys)) || (rc = alloc(&B.perm, n)) ||
        (rc = alloc(&B.block_sums, (size_t)scan_blocks)) || (rc = alloc(&B.tmp_cell, n)) ||
        (rc = alloc(&B.tmp_off, n)) || (rc = alloc(&B.diss_part, (size_t)nwarp_slots)) ||
        (rc = alloc(&B.peek_part, (size_t)nblocks * 12)) || (rc = alloc(&B.peek_vel, n)) ||
        (rc = alloc(&B.peek_force, n)) || (rc = alloc(&B.ctl, 1)) || (rc = alloc(&B.invperm, n)) ||
        (rc = alloc(&B.frac_part, (size_t)nwarp_slots)) || (rc = alloc(&B.ind_part, 6 * (size_t)nwarp_slots)) ||
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
  // launch shape of a variant's step kernel (the FP64-sum form has one shape)
  int block_of(int v) const { return sum64 ? 256 : variant_block<T>(v); }
  size_t smem_of(int v) const {
    if (sum64) return 0;
    // variant 11's bonded build stages the bond slot words too
    const size_t bond = (v == kAsyncHalfVariant && sizeof(T) == 4 && feat()) ? async_bond_smem(kWideBlock / 2, P.BMAX)
                                                                              : 0;
    return variant_smem<T>(v, P.prem != 0) + bond;
  }
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
        tdem::parallel_copy(host_stage + off, src[k], len[k] * sizeof(double));
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
    mirror_ok = false;
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
    StepHint nohint{};
    void* args[] = {&P, &B, &h, &hl, &cond_bits, &prim, &nohint};
    cudaKernelNodeParams kp = {};
    kp.func = reinterpret_cast<void*>(step_fn<T>(variant, kStep, feat(), sum64));
    kp.gridDim = dim3((unsigned)vgrid[variant]);
    kp.blockDim = dim3((unsigned)block_of(variant));
    kp.sharedMemBytes = (unsigned)smem_of(variant);
    kp.kernelParams = args;
    cudaGraphNode_t snode;
    if (P.BMAX > 0) {
      void* sargs[] = {&P, &B};
      cudaKernelNodeParams sk = {};
      if constexpr (sizeof(T) == 4) {
        sk.func = reinterpret_cast<void*>(&strain_kernel_async<T>);
        sk.gridDim = dim3((unsigned)sgrid);
        sk.blockDim = dim3(kStrainBlock);
        sk.sharedMemBytes = (unsigned)kStrainSmem;
      } else {
        sk.func = reinterpret_cast<void*>(&strain_kernel<T>);
        sk.gridDim = grid_n();
        sk.blockDim = dim3(kThreads);
      }
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
    if (P.BMAX <= 0) return;
    if constexpr (sizeof(T) == 4)
      strain_kernel_async<T><<<sgrid, kStrainBlock, kStrainSmem, s>>>(P, B);
    else
      strain_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B);
  }

  int prime(cudaStream_t s) {
    mirror_ok = false;
    launch_strain(s);
    step_fn<T>(variant, kPrime, feat(), sum64)<<<vgrid[variant], block_of(variant), smem_of(variant), s>>>(P, B, 0, 0, 0, 1, StepHint{});
    launch_rebuild(s);  // runs only if the prime step tripped the trigger
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    primed = true;
    return TDEM_OK;
  }

  int step(long long n, cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "step before set_state");
    if (n <= 0) {
      // no step: build the step graph for the current variant now, so that
      // the next call does not (instantiating it takes ~0.5 s)
      if (graph_on && !graph_failed && !exec && build_graph() != TDEM_OK) {
        graph_error = err;
        graph_failed = true;
        destroy_graphs();
        cudaGetLastError();
      }
      return TDEM_OK;
    }
    mirror_ok = false;  // rebuild decisions inside the step graph are the device's
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
      step_fn<T>(variant, kStep, feat(), sum64)<<<vgrid[variant], block_of(variant), smem_of(variant), s>>>(P, B, 0, 0, 0, 1, StepHint{});
      launch_rebuild(s);
    }
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  int peek(cudaStream_t s) {
    launch_strain(s);
    const int pr = primed ? 1 : 0;
    if (sum64 && feat())
      force_kernel<T, kPeek, true, true><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, pr, StepHint{});
    else if (sum64)
      force_kernel<T, kPeek, false, true><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, pr, StepHint{});
    else if (feat())
      force_kernel<T, kPeek, true><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, pr, StepHint{});
    else
      force_kernel<T, kPeek, false><<<grid_n(), kThreads, 0, s>>>(P, B, 0, 0, 0, pr, StepHint{});
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
      if (pos) tdem::parallel_copy(pos, host_stage, 2 * n * sizeof(double));
      if (vel) tdem::parallel_copy(vel, host_stage + 2 * n, 2 * n * sizeof(double));
      if (omega) tdem::parallel_copy(omega, host_stage + 4 * n, n * sizeof(double));
      if (force) tdem::parallel_copy(force, host_stage + 5 * n, 2 * n * sizeof(double));
      if (torque) tdem::parallel_copy(torque, host_stage + 7 * n, n * sizeof(double));
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
    refresh_mirror();
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
    const StepHint hint = mirror_ok ? StepHint{1, m_sp, m_lp, m_evals} : StepHint{};
    step_fn<T>(variant, kStep, feat(), sum64)<<<vgrid[variant], block_of(variant), smem_of(variant), s>>>(
        P, B, 0, 0, 0, 1, hint);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    // the launch's last block flips the state buffers and counts the evaluation
    m_sp ^= 1;
    ++m_evals;
    return TDEM_OK;
  }

  int rebuild_pending(cudaStream_t s) override {
    TDEM_CUDA_TRY(&err, cudaMemcpyAsync(host_ctl, B.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    refresh_mirror();
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
    mirror_ok = false;
    request_rebuild_kernel<<<1, 1, 0, s>>>(B.ctl);
    launch_rebuild(s);
    TDEM_CUDA_TRY(&err, cudaGetLastError());
    return TDEM_OK;
  }

  // Fragment label (smallest original id of the fragment) of every disc, in
  // original order, and the number of fragments (isolated discs included).
  int fragments(int* labels, long long* count, cudaStream_t s) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "fragments before set_state");
    const size_t n = (size_t)P.n;
    int *parent = nullptr, *label = nullptr, *out = nullptr, *changed = nullptr;
    unsigned long long* roots = nullptr;
    TDEM_CUDA_TRY(&err, cudaMallocAsync(&parent, n * sizeof(int), s));
    TDEM_CUDA_TRY(&err, cudaMallocAsync(&label, n * sizeof(int), s));
    TDEM_CUDA_TRY(&err, cudaMallocAsync(&out, n * sizeof(int), s));
    TDEM_CUDA_TRY(&err, cudaMallocAsync(&changed, sizeof(int), s));
    TDEM_CUDA_TRY(&err, cudaMallocAsync(&roots, sizeof(unsigned long long), s));
    cc_init_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, parent, label);
    int rc = TDEM_OK;
    bool done = P.BMAX == 0;
    // hooking with pointer jumping converges in a few rounds; the bound only
    // guards the host loop
    for (int it = 0; it < 256 && !done; ++it) {
      int h_changed = 0;
      TDEM_CUDA_TRY(&err, cudaMemsetAsync(changed, 0, sizeof(int), s));
      cc_hook_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, parent, changed);
      cc_compress_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, parent);
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(&h_changed, changed, sizeof(int), cudaMemcpyDeviceToHost, s));
      TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
      done = h_changed == 0;
    }
    if (!done) rc = tdem::fail(&err, TDEM_ERR_CUDA, "fragment labelling did not converge");
    unsigned long long h_roots = 0;
    if (!rc) {
      TDEM_CUDA_TRY(&err, cudaMemsetAsync(roots, 0, sizeof(unsigned long long), s));
      cc_label_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, parent, label, roots);
      cc_out_kernel<T><<<grid_n(), kThreads, 0, s>>>(P, B, parent, label, out);
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(labels, out, n * sizeof(int), cudaMemcpyDeviceToHost, s));
      TDEM_CUDA_TRY(&err, cudaMemcpyAsync(&h_roots, roots, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    }
    cudaFreeAsync(parent, s);
    cudaFreeAsync(label, s);
    cudaFreeAsync(out, s);
    cudaFreeAsync(changed, s);
    cudaFreeAsync(roots, s);
    TDEM_CUDA_TRY(&err, cudaStreamSynchronize(s));
    if (count) *count = (long long)h_roots;
    return rc;
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

  int set_wait_budget(long long cycles) override {
    if (cycles < 0) return tdem::fail(&err, TDEM_ERR_BADARG, "wait budget must be >= 0");
    P.wait_budget = cycles;
    destroy_graphs();  // the step graph holds the parameters by value
    return TDEM_OK;
  }

  // Time `steps` steps with every variant (advancing the simulation) and keep
  // the fastest. Per-particle arithmetic is identical in all variants.
  int autotune(int steps, cudaStream_t s, float* ms_out) override {
    if (!has_state) return tdem::fail(&err, TDEM_ERR_STATE, "autotune before set_state");
    mirror_ok = false;
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
    // a requested rebuild always ends by swapping both buffer sets
    m_sp ^= 1;
    m_lp ^= 1;
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

// Configuration checks shared by tdem_hm_create and the allocation-free entry
// point (static messages: no heap use). Null when the configuration is valid.
const char* hm_config_error(const tdem_hm_config* c) {
  if (c->n < 1) return "n out of range";
  if (c->max_neighbors < 1 || c->max_neighbors > kMaxSlots) return "max_neighbors must be in 1..24";
  if (!(c->inertia_factor > 0.0)) return "inertia_factor must be positive";
  if (c->max_bonds < 0 || c->max_bonds > kMaxBondSlots) return "max_bonds must be in 0..8";
  if (c->max_bonds > 0 && (!(c->bond_kn > 0) || !(c->bond_ks >= 0) || !(c->bond_damping >= 0) ||
                           !(c->breaking_strain > 0) || !(c->shear_breaking_strain > 0)))
    return "invalid bond stiffness, damping or break strain";
  if (!(c->indenter_radius >= 0)) return "indenter_radius must be >= 0";
  // cell ids pack cx | cy << 16, and the key space is (tiles_x * tiles_y) << 10
  if (c->ncx < 1 || c->ncy < 1 || c->ncx > 32768 || c->ncy > 32768) return "cell grid must be 1..32768 per axis";
  if (!(c->cell > 0) || !(c->skin >= 0) || !(c->dt > 0) || !(c->young > 0) || !(c->poisson > -1.0) ||
      !(c->poisson < 0.5) || !(c->restitution > 0) || !(c->restitution <= 1) || !(c->mu >= 0) ||
      !(c->mu_wall >= 0))
    return "invalid material, cell or time-step parameter";
  if (c->precision != 32 && c->precision != 64) return "precision must be 32 or 64";
  if (c->sum_precision != 0 && c->sum_precision != 32 && c->sum_precision != 64)
    return "sum_precision must be 0, 32 or 64";
  if (c->position_remainder != 0 && c->position_remainder != 1) return "position_remainder must be 0 or 1";
  return nullptr;
}

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
  if (const char* why = hm_config_error(c)) return tdem::fail(err, TDEM_ERR_BADARG, why);
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

int tdem_hm_fragments(tdem_hm* h, int32_t* labels, int64_t* count, void* stream) {
  if (!h || !labels) return TDEM_ERR_BADARG;
  long long c = 0;
  const int rc = h->e->fragments(labels, &c, reinterpret_cast<cudaStream_t>(stream));
  if (count) *count = (int64_t)c;
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

int tdem_hm_set_wait_budget(tdem_hm* h, int64_t cycles) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->set_wait_budget((long long)cycles);
}

int tdem_hm_autotune(tdem_hm* h, int steps, float* ms_out, void* stream) {
  if (!h || steps < 1) return TDEM_ERR_BADARG;
  return h->e->autotune(steps, reinterpret_cast<cudaStream_t>(stream), ms_out);
}

int tdem_hm_use_graph(tdem_hm* h, int on) {
  if (!h) return TDEM_ERR_BADARG;
  return h->e->use_graph(on);
}

}  // extern "C"

namespace {

// The per-contact law of the step kernel (contact_law, with the effective
// radius and mass formed as pair_force forms them) on rows of pair states:
// in row k (16 doubles): overlap delta, unit normal (x, y) from a to b, r_a,
// r_b, a's vx, vy, omega, b's vx, vy, omega, 1/m_a, 1/m_b, history xi (x, y)
// in a's orientation, one unused; out row k (8 doubles): force on a (x, y),
// n x F_a, updated history (x, y), dissipated energy, Hertz and tangential
// spring energies. A pair without overlap, or of two clamped discs, reports
// zeros (its history resets).
template <class T>
__global__ void contact_law_kernel(Params<T> P, long long count, const double* in, double* out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const double* r = in + 16 * k;
  double* o = out + 8 * k;
  const T delta = (T)r[0], nx = (T)r[1], ny = (T)r[2], ra = (T)r[3], rb = (T)r[4];
  const V4<T> va{(T)r[5], (T)r[6], (T)r[7], (T)r[11]}, vb{(T)r[8], (T)r[9], (T)r[10], (T)r[12]};
  if (!(delta > T(0)) || !(va.w + vb.w > T(0))) {
    for (int q = 0; q < 8; ++q) o[q] = 0.0;
    return;
  }
  T reff, meff;
  pair_effective<T>(ra, rb, va.w, vb.w, reff, meff);
  const PairOut<T> c = contact_law<T>(P, delta, nx, ny, reff, meff, ra, rb, va, vb, V2<T>{(T)r[13], (T)r[14]});
  o[0] = (double)c.fx;
  o[1] = (double)c.fy;
  o[2] = (double)c.cr;
  o[3] = (double)c.xi.x;
  o[4] = (double)c.xi.y;
  o[5] = (double)c.diss;
  o[6] = (double)c.un;
  o[7] = (double)c.ut;
}

template <class T>
int contact_law_run(const tdem_hm_config& cfg, long long count, const double* in, double* out, cudaStream_t s) {
  Params<T> P{};
  make_params<T>(cfg, 1, P);
  double *din = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&din, (size_t)count * 16 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)count * 8 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, (size_t)count * 16 * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    contact_law_kernel<T><<<(unsigned)((count + 127) / 128), 128, 0, s>>>(P, count, din, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)count * 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(din);
  cudaFree(dout);
  return e == cudaSuccess ? TDEM_OK : TDEM_ERR_CUDA;
}

}  // namespace

extern "C" {

int tdem_hm_contact_law(const tdem_hm_config* cfg, int64_t count, const double* in, double* out, void* stream) {
  g_hm_create_error.clear();
  if (!cfg || (count > 0 && (!in || !out)) || count < 0)
    return tdem::fail(&g_hm_create_error, TDEM_ERR_BADARG, "null argument or negative count");
  if (!(cfg->dt > 0) || !(cfg->young > 0) || !(cfg->poisson > -1.0) || !(cfg->poisson < 0.5) ||
      !(cfg->restitution > 0) || !(cfg->restitution <= 1) || !(cfg->mu >= 0))
    return tdem::fail(&g_hm_create_error, TDEM_ERR_BADARG, "invalid material or time-step parameter");
  if (cfg->precision != 32 && cfg->precision != 64)
    return tdem::fail(&g_hm_create_error, TDEM_ERR_BADARG, "precision must be 32 or 64");
  if (count == 0) return TDEM_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int rc = cfg->precision == 32 ? contact_law_run<float>(*cfg, (long long)count, in, out, s)
                                      : contact_law_run<double>(*cfg, (long long)count, in, out, s);
  if (rc) return tdem::fail(&g_hm_create_error, rc, "CUDA error in the contact-law evaluation");
  return TDEM_OK;
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
// For callers that must not allocate device memory: plug-ins whose host
// application owns and budgets all device memory, and real-time coupling
// loops where an allocation's latency or failure is not acceptable. The
// scratch lives in one file-scope device array that every GPU loading this
// library holds until the process exits. Its device address is resolved on a
// device's first call and kept for the process (a device reset in between
// would leave it stale).
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
int noalloc_fail(char* buf, size_t len, int code, const char* fmt, long long a = 0, long long b = 0,
                 const char* text = nullptr) {
  if (buf && len) {
    if (text)
      snprintf(buf, len, fmt, text);
    else
      snprintf(buf, len, fmt, a, b);
  }
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
  // the engine's own configuration checks (grid, material, skin, dt, friction)
  if (const char* why = hm_config_error(cfg)) return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG, "%s", 0, 0, why);
  if (cfg->max_bonds != 0 || cfg->indenter_radius != 0.0)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG,
                        "the allocation-free path evaluates contacts, walls and gravity only: max_bonds and "
                        "indenter_radius must be 0");
  // the key count in 64-bit before any index arithmetic depends on it
  const long long keys = (long long)((cfg->ncx + 31) / 32) * (long long)((cfg->ncy + 31) / 32) * 1024LL;
  if (keys > kNoAllocMaxKeys)
    return noalloc_fail(err_buf, err_len, TDEM_ERR_BADARG,
                        "the allocation-free path holds cell grids up to 256 x 256 cells; this grid is %lld x %lld",
                        (long long)cfg->ncx, (long long)cfg->ncy);
  Params<float> P{};
  make_params<float>(*cfg, kNoAllocSlots, P);
  P.BMAX = 0;  // contacts, walls and gravity only: no bond slots live in the scratch
  P.irad = 0.0f;
  P.load_cap = 0;
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
  force_kernel<float, kPeek, false><<<nb, kThreads, 0, s>>>(P, B, 0, 0, 0, 0, StepHint{});
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
