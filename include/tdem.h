/*
 * tdem.h - C ABI of the GB300 (sm_103a) 2-D DEM step library, libtdem_sm103.so.
 *
 * Plain C: opaque handles, plain pointers and sizes. Device pointers are CUDA
 * device addresses (for example torch.Tensor.data_ptr() of a contiguous CUDA
 * tensor); host pointers are ordinary (ideally pinned) host memory. A
 * `void* stream` is a cudaStream_t (NULL = the legacy default stream).
 *
 * Every function returns an int status: TDEM_OK (0) or one of the TDEM_ERR_*
 * codes below; the text of the last error of a handle is available from
 * tdem_last_error(). Handles are not re-entrant: one handle per stream.
 *
 * Two engines sit behind this ABI:
 *
 *  1. "icedem": the reference mode. It reproduces, in FP64, the step of the
 *     reference's `IceDEM` (src/tensordem/dem.py:75-624): central-force bonds
 *     on the square+diagonal lattice, tensile and objective-shear breakage,
 *     linear penalty contacts with a no-tension clamp, a circular indenter or
 *     a polyline hull, linear drag, semi-implicit Euler and the accounting
 *     ledger. The state arrays are owned by the caller (the Python drop-in
 *     keeps them as torch tensors) and passed on every call.
 *
 *  2. "hm": the Hertz-Mindlin mode, a 2-D disc engine: cell-list
 *     contact detection with a Verlet skin, Hertz normal + Tsuji dashpot,
 *     Mindlin tangential spring with Coulomb cap and per-contact history,
 *     bonded-particle normal/shear springs with irreversible tensile and
 *     objective-shear breakage, planar walls, a circular indenter, gravity and
 *     velocity-Verlet. FP32 per-contact arithmetic on FP32 offsets from an
 *     integer cell origin; compensated (float-float) per-particle sums; FP64
 *     ledger. Its state lives in the handle, in HBM.
 */
#ifndef TDEM_H_
#define TDEM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TDEM_OK = 0,
  TDEM_ERR_BADARG = 1,    /* invalid argument: maps to ValueError */
  TDEM_ERR_CUDA = 2,      /* a CUDA runtime call failed: RuntimeError */
  TDEM_ERR_NONFINITE = 3, /* non-finite state after a step: FloatingPointError */
  TDEM_ERR_CAPACITY = 4,  /* a fixed-capacity buffer overflowed: RuntimeError */
  TDEM_ERR_STATE = 5      /* call out of order (e.g. no state uploaded) */
};

/* Library version, for a loader's sanity check. */
int tdem_version(void);

/* ========================================================================
 * 1. Reference mode ("icedem")
 * ====================================================================== */

typedef struct tdem_icedem tdem_icedem;

/* Constant configuration of one IceDEM instance. Field meaning follows the
 * reference's DEMConfig (src/tensordem/dem.py:17-72); `mass` is the disc mass
 * rho*pi*r^2*t and `dt` the resolved step (config.dt or recommended_dt). */
typedef struct {
  int32_t n;                /* number of discs, 2 <= n <= tdem_icedem_max_discs() */
  double radius;
  double mass;
  double bond_stiffness;
  double contact_stiffness;
  double breaking_strain;
  double shear_breaking_strain;
  double contact_damping;
  double drag;
  double tool_radius;
  double dt;
  double tool_start[2];     /* dem.py:146-150 */
  double tool_velocity[2];  /* dem.py:151-153 */
  int32_t hull_vertices;    /* 0: circular tool; >= 2: polyline hull (dem.py:154-169) */
  const double* hull_profile_host; /* (hull_vertices, 2) host, local hull vertices */
  double hull_start[2];
  double hull_velocity[2];
} tdem_icedem_config;

/* Caller-owned state, device pointers, passed on every call. Pair-indexed
 * arrays use the reference's all-pairs order: pair p = (i, j), i < j, in the
 * row-major order of triu_indices(n, n, 1) (dem.py:116-118). */
typedef struct {
  double* positions;             /* (n, 2) m */
  double* velocities;            /* (n, 2) m/s */
  const double* initial_positions; /* (n, 2) m */
  const uint8_t* fixed;          /* (n,) bool */
  uint8_t* alive;                /* (P,) bool, P = n(n-1)/2 */
  uint8_t* failure_mode;         /* (P,) 0 intact, 1 tensile, 2 shear, 3 both */
  double* failure_time_s;        /* (P,) */
  double* failure_extension_m;   /* (P,) */
  double* failure_energy_J;      /* (P,) */
} tdem_icedem_state;

/* Ledger slots of tdem_icedem_read_ledger / tdem_icedem_write_ledger. The
 * first 13 are the reference's `accounting` dict (dem.py:139-144) in this
 * order; the rest mirror `last_step` (dem.py:372-376) and diagnostics. */
enum {
  TDEM_L_EXTERNAL_WORK = 0, TDEM_L_FRACTURE_RELEASE, TDEM_L_CONTACT_ACQUIRED,
  TDEM_L_TOOL_WORK, TDEM_L_DAMPING_DISSIPATION,
  TDEM_L_EXTERNAL_IMPULSE_X, TDEM_L_EXTERNAL_IMPULSE_Y,
  TDEM_L_SUPPORT_IMPULSE_X, TDEM_L_SUPPORT_IMPULSE_Y,
  TDEM_L_DRAG_IMPULSE_X, TDEM_L_DRAG_IMPULSE_Y,
  TDEM_L_TOOL_IMPULSE_X, TDEM_L_TOOL_IMPULSE_Y,
  TDEM_L_LAST_SUPPORT_X = 13, TDEM_L_LAST_SUPPORT_Y,
  TDEM_L_LAST_REACTION_X, TDEM_L_LAST_REACTION_Y,
  TDEM_L_LAST_EXTERNAL_X, TDEM_L_LAST_EXTERNAL_Y,
  TDEM_L_LAST_EXTERNAL_WORK, TDEM_L_LAST_EXTERNAL_MOMENT,
  TDEM_L_LAST_TIME_START, TDEM_L_LAST_TIME_END,
  TDEM_L_DAMPING_POWER, TDEM_L_TOOL_POWER,
  TDEM_L_MIN_BREAK_MARGIN, /* min over steps/alive bonds of the relative distance to a threshold */
  TDEM_L_COUNT = 32
};

/* Largest disc count of one reference-mode instance (one CTA holds it). */
int tdem_icedem_max_discs(void);

/* Build the instance: bond topology from `initial_positions_host` ((n,2),
 * bonds where |x_j - x_i| <= 2 r sqrt(2) (1 + 1e-10), dem.py:119-124), the
 * per-disc bond lists in the reference's accumulation order, and the constant
 * pseudo-inverse of each disc's bond covariance (dem.py:194-202).
 * Replaces IceDEM.__init__ (dem.py:86-169). */
int tdem_icedem_create(const tdem_icedem_config* cfg, const double* initial_positions_host,
                       tdem_icedem** out);
void tdem_icedem_destroy(tdem_icedem* h);

/* Number of bonds found at create time and their pair indices (host out, int64). */
int tdem_icedem_num_bonds(const tdem_icedem* h);
int tdem_icedem_bond_pairs(const tdem_icedem* h, int64_t* out_pair_index_host);

/* Per-bond central-spring stiffness (host, one value per bond in bond order,
 * each finite, > 0 and <= cfg.bond_stiffness). Every later evaluation adds,
 * after the base force, (k_b - k) (d - L0) n on each surviving bond and books
 * the actual spring energy of a bond when it breaks. Replaces the force and
 * energy overrides of CalibratedIceDEM (src/tensordem/calibrated_dem.py:11-93). */
int tdem_icedem_set_bond_stiffness(tdem_icedem* h, const double* k_host, int count);

/* One force evaluation at `time`: commits breaks and their ledger entries and
 * writes the total force (n,2) and the ice-on-tool reaction (2) to device
 * buffers. `loads` is an optional (n,2) device array of external nodal
 * forces (NULL = none). Replaces IceDEM.forces (dem.py:226-345). */
int tdem_icedem_forces(tdem_icedem* h, const tdem_icedem_state* st, const double* loads,
                       double time, double* out_force, double* out_reaction, void* stream);

/* `n_steps` semi-implicit Euler steps from `time` in one launch (loads, if
 * given, are held over all of them). Replaces IceDEM.step (dem.py:347-382).
 * Returns TDEM_ERR_NONFINITE (after finishing the offending step, as the
 * reference does) when the state stops being finite; the call synchronizes
 * `stream` to read that status. */
int tdem_icedem_step(tdem_icedem* h, const tdem_icedem_state* st, const double* loads,
                     int n_steps, double time, void* stream);

/* Steps completed by the last tdem_icedem_step call (less than requested only
 * when it stopped on a non-finite state). */
int tdem_icedem_steps_done(const tdem_icedem* h);

/* Fragments of the state: connected components of the intact bonds given
 * by the per-pair alive flags (P,) bool (device), isolated discs included.
 * labels_host[k] (n ints) = the smallest disc id of disc k's fragment.
 * Replaces the component search of IceDEM.fragments
 * (src/tensordem/dem.py:462-484). Synchronizes `stream`. */
int tdem_icedem_fragments(tdem_icedem* h, const void* alive, int32_t* labels_host, void* stream);

/* Stored mechanical energy of the state (positions, velocities (n,2) FP64 and
 * the per-pair alive flags (P,) bool, device arrays) with the tool at `time`:
 * out_host[0..4] = kinetic, intact-bond springs (per-bond stiffness when
 * set), penalty energy of overlapping pairs that are not intact bonds, tool
 * penalty energy, their sum (J). Replaces IceDEM.mechanical_energy
 * (src/tensordem/dem.py:603-624) and its per-bond-stiffness form
 * (src/tensordem/calibrated_dem.py:79-93). Synchronizes `stream`. */
int tdem_icedem_energy(tdem_icedem* h, const double* positions, const double* velocities, const void* alive,
                       double time, double* out_host, void* stream);

/* The TDEM_L_COUNT ledger doubles copied into a device buffer, ordered on
 * `stream` (no synchronization): lets a caller record diagnostics rows on the
 * device, as the dem-2d command's history does (src/tensordem/cli.py:69-105). */
int tdem_icedem_ledger_to_device(tdem_icedem* h, double* out_device, void* stream);

/* Ledger transfer (host doubles, up to TDEM_L_COUNT). Synchronizes `stream`. */
int tdem_icedem_read_ledger(tdem_icedem* h, double* out_host, int count, void* stream);
int tdem_icedem_write_ledger(tdem_icedem* h, const double* in_host, int count, void* stream);

/* Text of the last error of `h` (or of the last failed create when h is NULL). */
int tdem_icedem_last_error(const tdem_icedem* h, char* buf, size_t len);

/* ========================================================================
 * 2. Hertz-Mindlin mode ("hm"): 2-D Hertz-Mindlin discs
 * ====================================================================== */

typedef struct tdem_hm tdem_hm;

/* Configuration. The box is [0, ncx*cell] x [0, ncy*cell]; walls sit on its
 * edges (bit 0 left x=0, bit 1 right, bit 2 bottom y=0, bit 3 top). `cell`
 * must be >= 2 r_max + skin. Material: E, nu, restitution (Tsuji damping),
 * particle and wall friction. Contact law as the reference's Hertz-Mindlin
 * pieces: src/tensordem/scale_ceiling/kernel.py:277-401,
 * src/tensordem/hertz_mindlin.py:94-176, src/tensordem/granular2d/engine.py:458-503. */
typedef struct {
  int32_t n;              /* particles */
  int32_t precision;      /* 32: FP32 contacts, compensated sums; 64: plain FP64 */
  int32_t max_neighbors;  /* candidate slots per particle, 1..24 */
  int32_t walls;          /* wall bit mask */
  int32_t ncx, ncy;       /* cell grid */
  double cell;            /* cell edge (m) */
  double skin;            /* Verlet skin (m) */
  double dt;              /* time step (s) */
  double young, poisson, restitution, mu, mu_wall;
  double gravity[2];      /* m/s^2 */
  double inertia_factor;  /* I = inertia_factor * m * r^2 (0.5 for uniform discs) */
  /* bonded-particle model (max_bonds == 0: none; bonds come from tdem_hm_set_bonds) */
  int32_t max_bonds;      /* bond slots per disc, 0..8 */
  double bond_kn, bond_ks;  /* bond normal / shear stiffness (N/m) */
  double bond_damping;    /* damping ratio zeta: c = 2 zeta sqrt(k m*) */
  double breaking_strain; /* tensile (d - L0)/L0 threshold, times the bond's strength */
  double shear_breaking_strain; /* objective shear threshold, times the strength */
  /* rigid circular indenter (radius 0: none): Hertz normal + dashpot, frictionless */
  double indenter_center[2];   /* at t = 0 (m) */
  double indenter_velocity[2]; /* m/s */
  double indenter_radius;      /* m */
  int32_t load_capacity;  /* evaluations whose indenter reaction is recorded */
  int32_t sum_precision;  /* FP32 engines: 64 sums each particle's force and
                             torque terms in FP64; 0 or 32: compensated FP32
                             (float-float) sums. FP64 engines sum in FP64. */
  int32_t position_remainder; /* FP32 engines: 1 keeps each position's FP32
                             rounding remainder (one FP32 pair per disc, 16 more
                             bytes per disc and step), so that positions
                             integrate to about 48 bits and the energy ledger
                             closes as in FP64 before any break; 0: plain FP32
                             offsets. Ignored by FP64 engines and by the
                             allocation-free entry point. */
} tdem_hm_config;

/* Ledger slots of tdem_hm_read_ledger (J unless noted). */
enum {
  TDEM_HM_L_KINETIC = 0,     /* translational + rotational */
  TDEM_HM_L_POTENTIAL = 1,   /* gravitational, -sum m g.x */
  TDEM_HM_L_HERTZ = 2,       /* normal elastic 0.4 F_el delta */
  TDEM_HM_L_TANGENTIAL = 3,  /* tangential spring 0.5 S_t |xi|^2 */
  TDEM_HM_L_TOTAL = 4,       /* sum of the above + dissipated */
  TDEM_HM_L_DISSIPATED = 5,  /* cumulative dashpot + Coulomb slip loss */
  TDEM_HM_L_EVALS = 6,       /* committed force evaluations */
  TDEM_HM_L_REBUILDS = 7,    /* neighbour-list rebuilds */
  TDEM_HM_L_MAX_NEIGHBORS = 8, /* largest candidate count at the last rebuild */
  TDEM_HM_L_STATUS = 9,      /* device status bits */
  TDEM_HM_L_GRAPH = 10,      /* 1 when steps run as conditional CUDA graphs */
  TDEM_HM_L_VARIANT = 11,    /* step-kernel variant in use */
  TDEM_HM_L_BOND_ELASTIC = 12, /* stored bond energy of intact bonds */
  TDEM_HM_L_FRACTURE = 13,   /* cumulative spring energy released by breaks */
  TDEM_HM_L_TOOL_WORK = 14,  /* cumulative work of the indenter on the discs */
  TDEM_HM_L_BROKEN = 15,     /* bonds broken so far */
  TDEM_HM_L_COUNT = 16
};

/* Allocate the engine (all device buffers sized for n). Replaces the
 * reference engines' constructors: FloeBed.__init__
 * (src/tensordem/scale_ceiling/kernel.py:147-197) and DiskSystem.__init__
 * (src/tensordem/granular2d/engine.py:147-211). */
int tdem_hm_create(const tdem_hm_config* cfg, tdem_hm** out);
void tdem_hm_destroy(tdem_hm* h);

/* Upload a state in original particle order (FP64: positions (n,2),
 * velocities (n,2), omega (n), radius (n), mass (n), moment of inertia (n));
 * host=1: host pointers (staged through pinned memory), host=0: device
 * pointers. Builds the first neighbour list (cell list, kernel.py:230-266,
 * src/tensordem/scale_ceiling/search.py:60-162). */
int tdem_hm_set_state(tdem_hm* h, const double* pos, const double* vel, const double* omega,
                      const double* radius, const double* mass, const double* inertia, int host,
                      void* stream);

/* Advance n velocity-Verlet steps (FloeBed.step, kernel.py:410-419), list
 * rebuilds and history remap included (kernel.py:230-274). Asynchronous:
 * check tdem_hm_status afterwards. n_steps == 0 steps nothing and builds the
 * step graph for the current variant if it is not built yet (the first
 * stepping call after creation or a variant change otherwise pays that,
 * about half a second). */
int tdem_hm_step(tdem_hm* h, int64_t n_steps, void* stream);

/* Integer-time state in original order: positions, velocities, omega, total
 * force (incl. gravity), torque; any output may be NULL. host=1: host
 * pointers (synchronizes), host=0: device pointers. */
int tdem_hm_read_state(tdem_hm* h, double* pos, double* vel, double* omega, double* force,
                       double* torque, int host, void* stream);

/* Energy ledger and counters (TDEM_HM_L_*) into host doubles; synchronizes.
 * Mirrors FloeBed.energy_ledger (kernel.py:483-487) plus the dissipation
 * ledger of DiskSystem (granular2d/engine.py:576-588). */
int tdem_hm_read_ledger(tdem_hm* h, double* out_host, int count, void* stream);

/* Bonds between discs of the uploaded state (call after tdem_hm_set_state,
 * before the first step): `pairs` (count, 2) original ids and a strength
 * factor per bond (host arrays). Rest vectors are the current positions'
 * differences; each disc's bond covariance pseudo-inverse is precomputed
 * (src/tensordem/dem.py:119-129, 194-202). Replaces the bond build of
 * IceDEM.__init__ for arbitrary lattices (hexagonal sheets included). */
int tdem_hm_set_bonds(tdem_hm* h, const int32_t* pairs, const double* strength, int64_t count, void* stream);

/* Bond states, one entry per bond as original ids (lo, hi) into pairs
 * ((capacity, 2) int32, host) and (mode, evaluation of failure) into state
 * ((capacity, 2) int32): mode 0 intact, 1 tensile, 2 shear, 3 both; -1 for an
 * intact bond's evaluation (the reference's fracture ledger, dem.py:131-136). */
int tdem_hm_read_bonds(tdem_hm* h, int32_t* pairs, int32_t* state, int64_t capacity, int64_t* count,
                       void* stream);

/* Indenter reaction (ice on indenter, x, y) of each committed evaluation,
 * up to load_capacity evaluations, into out ((capacity, 2) double, host). */
int tdem_hm_read_load(tdem_hm* h, double* out, int64_t capacity, int64_t* count, void* stream);

/* Fragments: connected components of the intact bonds (isolated discs are
 * fragments of one). labels (n, host int32, original order) receives each
 * disc's fragment label, the smallest original id in its fragment; count the
 * number of fragments. Replaces IceDEM.fragments' host search
 * (src/tensordem/dem.py:462-484) with a device union-find. Synchronizes. */
int tdem_hm_fragments(tdem_hm* h, int32_t* labels, int64_t* count, void* stream);

/* Synchronize and map the device status: TDEM_ERR_NONFINITE, TDEM_ERR_CAPACITY. */
int tdem_hm_status(tdem_hm* h, void* stream);

/* Current candidate pairs as original ids (i < j), for verification against a
 * brute-force search (tests/test_scale_ceiling_dem.py:41-50). Writes up to
 * `capacity` pairs to out_host ((capacity, 2) int32) and the total to *count. */
int tdem_hm_read_pairs(tdem_hm* h, int32_t* out_host, int64_t capacity, int64_t* count, void* stream);

/* Rebuild the neighbour list now (sort by cell, candidates, history remap),
 * as FloeBed.build_neighbours(keep_state=True) does
 * (src/tensordem/scale_ceiling/kernel.py:230-266). */
int tdem_hm_rebuild(tdem_hm* h, void* stream);

/* Stored tangential history of every pair with a non-zero value: original ids
 * (lo, hi) into pairs ((capacity, 2) int32, host) and the displacement of lo
 * relative to hi into xi ((capacity, 2) double, host). The reference keeps the
 * same state keyed by i*N+j (src/tensordem/granular2d/engine.py:388-396). */
int tdem_hm_read_history(tdem_hm* h, int32_t* pairs, double* xi, int64_t capacity, int64_t* count,
                         void* stream);

/* One step as a single plain launch of the step kernel, with no rebuild:
 * for callers that time the kernel alone (a list rebuild must follow when
 * tdem_hm_rebuild_pending says so, before the next step). */
int tdem_hm_step_kernel(tdem_hm* h, void* stream);

/* Synchronize `stream`; 1 if the neighbour list must be rebuilt before the
 * next step (then call tdem_hm_rebuild), 0 if not, negative on error. */
int tdem_hm_rebuild_pending(tdem_hm* h, void* stream);

/* Step-kernel variants (launch shapes) and the autotuner that picks one by
 * timing `steps` steps of each on the live state (the simulation advances by
 * tdem_hm_num_variants() * (steps + 2) steps). ms_out (optional, host) gets
 * one time per variant. All variants compute bit-identical particle states. */
int tdem_hm_num_variants(void);
int tdem_hm_set_variant(tdem_hm* h, int variant);
int tdem_hm_get_variant(const tdem_hm* h);
/* SM clock cycles a bounded wait of the bulk-copy step kernels (variants 4-6)
 * may take before the kernel records a timeout, drains its copies in flight
 * and returns (default ~2e9, about a second). For tests of the failure path:
 * a budget of 0 makes each wait a single non-blocking probe of the copy it
 * waits for, so the waits run out; the next status check then fails
 * with TDEM_ERR_CUDA, and the engine recovers with set_state. No counterpart
 * in the reference (it has no device waits). */
int tdem_hm_set_wait_budget(tdem_hm* h, int64_t cycles);
int tdem_hm_autotune(tdem_hm* h, int steps, float* ms_out, void* stream);

/* Allocation-free contact forces. No counterpart in the reference: it exists
 * for callers that cannot allocate device memory, such as plug-ins whose host
 * application owns and budgets all device memory, and real-time coupling
 * loops in which an allocation's latency or failure cannot be accepted.
 *
 * One Hertz-Mindlin force evaluation of `cfg->n` discs given in original order
 * as device arrays (positions (n,2), velocities (n,2), omega, radius, mass,
 * inertia; FP64): cell list, candidate lists and the contact, wall and gravity
 * forces with zero tangential history, as tdem_hm_set_state followed by
 * tdem_hm_read_state would report them. Writes the total force (n,2) and
 * torque (n) to the device arrays out_force / out_torque. FP32 only.
 *
 * It calls no cudaMalloc or cudaFree: its scratch is one 8 MiB device array
 * inside this library, which every GPU that loads the library holds until the
 * process exits. Limits: n <= 16384 discs, grids up to 256 x 256 cells, at
 * most 8 candidate partners per disc; larger inputs are rejected with
 * TDEM_ERR_BADARG (or TDEM_ERR_CAPACITY for a crowded disc) and a message in
 * err_buf (optional, err_len bytes); the configuration passes the same checks
 * as tdem_hm_create, and max_bonds and indenter_radius must be 0 (contacts,
 * walls and gravity only). The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress) and keeps it for the process: make
 * that first call before any stream capture, and do not reset the device
 * (cudaDeviceReset) between calls. All calls share the one array, which keeps
 * the last call's contents (each call clears what must start at zero): calls
 * that overlap on the GPU, on any streams or threads, race. The call
 * synchronizes `stream` to read the evaluation's status. */
int tdem_hm_contact_forces_noalloc(const tdem_hm_config* cfg, const double* pos, const double* vel,
                                   const double* omega, const double* radius, const double* mass,
                                   const double* inertia, double* out_force, double* out_torque,
                                   char* err_buf, size_t err_len, void* stream);

/* The Hertz-Mindlin contact law on its own: the per-contact arithmetic of
 * the step kernel (the same device function) applied to `count` pair states,
 * in the engine's precision (cfg->precision) with cfg's material (young,
 * poisson, restitution, mu, dt; the grid fields are not used). Replaces the
 * reference's contact-law helpers: the Hertz normal force with the Tsuji
 * dashpot (src/tensordem/scale_ceiling/kernel.py:300-310), the Mindlin
 * tangential spring with the Coulomb cap and state projection
 * (src/tensordem/hertz_mindlin.py:118-176) and the history increment
 * (src/tensordem/contact_tangential.py:377-417).
 *
 * in (host, count x 16 doubles per row): overlap delta, unit normal (x, y)
 * from a to b, r_a, r_b, v_a (x, y), omega_a, v_b (x, y), omega_b, 1/m_a,
 * 1/m_b, stored history xi (x, y) in a's orientation, 1 unused. out (host,
 * count x 8 per row): force on a (x, y), n x F_a (the torque on a is r_a
 * times it), updated history (x, y), dissipated energy of the step, Hertz
 * energy, spring energy. A pair without overlap (delta <= 0), or of two
 * clamped discs (1/m_a + 1/m_b = 0), reports zeros: its history resets.
 * Synchronizes `stream`. */
int tdem_hm_contact_law(const tdem_hm_config* cfg, int64_t count, const double* in, double* out, void* stream);

/* 1 (default): steps run as one conditional CUDA graph launch; 0: plain launches. */
int tdem_hm_use_graph(tdem_hm* h, int on);

int tdem_hm_last_error(const tdem_hm* h, char* buf, size_t len);

/* ========================================================================
 * 3. Batched ragged engine ("batch"): many independent Hertz-Mindlin solves
 * ====================================================================== */

/* Many independent solves of uneven sizes (each described by a
 * tdem_hm_config and its own state, material, walls, bonds and indenter)
 * packed into one sorted SoA and advanced together: one persistent step
 * kernel per step, one conditional CUDA graph launch per step block. Each
 * instance owns a contiguous range of cell keys and so a contiguous range of
 * the sorted arrays, cut into 32-particle tiles that a warp processes with
 * the instance's parameters. Per-instance ledgers are summed in tile order:
 * an instance's result does not depend on the other instances in the batch
 * except through the (shared) rebuild schedule; with rebuild_every > 0 and no
 * displacement-triggered rebuild the results are bit-identical alone and in
 * any mix.
 *
 * The reference runs one `IceDEM` / engine object per solve
 * (src/tensordem/dem.py:75); these entry points replace a loop over such
 * objects (src/tensordem/sensitivity.py:36-75 runs that loop). */
typedef struct tdem_batch tdem_batch;

typedef struct {
  int32_t precision;         /* 32: FP32 contacts, compensated sums, FP64 ledger; 64: plain FP64 */
  int32_t max_neighbors;     /* candidate slots per particle, 1..24 */
  int32_t max_bonds;         /* bond slots per particle, 0..8 */
  int32_t max_instances;     /* instance slots */
  int64_t particle_capacity; /* particles resident at once (live + retired awaiting compaction) */
  int64_t key_capacity;      /* cell keys over all instances (an instance takes ncx * ncy) */
  int32_t rebuild_every;     /* 0: rebuild on the displacement bound only; k > 0: also every k steps */
  int32_t position_remainder; /* FP32: 1 keeps each position's rounding remainder (see tdem_hm_config) */
} tdem_batch_config;

/* Ledger slots of tdem_batch_read: TDEM_HM_L_* (per instance; EVALS counts
 * the instance's own evaluations) followed by these. */
enum {
  TDEM_BATCH_L_PEAK_LOAD = 16,   /* max over evaluations of |indenter reaction| (N) */
  TDEM_BATCH_L_PEAK_EVAL = 17,   /* instance evaluation index of that maximum */
  TDEM_BATCH_L_REACTION_X = 18,  /* indenter reaction of the last evaluation (N) */
  TDEM_BATCH_L_REACTION_Y = 19,
  TDEM_BATCH_L_COUNT = 20
};

/* Slots of tdem_batch_info. */
enum {
  TDEM_BATCH_I_LIVE_PARTICLES = 0, TDEM_BATCH_I_LIVE_INSTANCES, TDEM_BATCH_I_EVALS, TDEM_BATCH_I_REBUILDS,
  TDEM_BATCH_I_TILES, TDEM_BATCH_I_PARTICLE_CAPACITY, TDEM_BATCH_I_BYTES, TDEM_BATCH_I_KEY_HI,
  TDEM_BATCH_I_STATUS, TDEM_BATCH_I_VARIANT, TDEM_BATCH_I_GRAPH, TDEM_BATCH_I_MAX_NEIGHBORS,
  TDEM_BATCH_I_COUNT
};

/* Device bytes a batch with this configuration allocates (admission by HBM
 * footprint sizes its capacities with this). */
int tdem_batch_bytes(const tdem_batch_config* cfg, int64_t* bytes);

/* Allocate every device buffer for the capacities in one allocation. */
int tdem_batch_create(const tdem_batch_config* cfg, tdem_batch** out);
void tdem_batch_destroy(tdem_batch* h);

/* Admit one instance: its configuration (`n`, grid, cell, skin, dt, material,
 * walls, gravity, bond law, indenter; `precision`, `max_neighbors`,
 * `max_bonds` and `load_capacity` are the batch's), its state in host FP64
 * arrays in local order (as tdem_hm_set_state), and optional bonds (pairs of
 * local ids with strength factors). The instance joins at the next step
 * boundary; its first step primes velocity-Verlet. Writes its id.
 * Synchronizes `stream`. TDEM_ERR_CAPACITY when particles, keys or slots
 * are exhausted. */
int tdem_batch_admit(tdem_batch* h, const tdem_hm_config* inst, const double* pos, const double* vel,
                     const double* omega, const double* radius, const double* mass, const double* inertia,
                     const int32_t* bond_pairs, const double* bond_strength, int64_t n_bonds, int32_t* out_id,
                     void* stream);

/* Advance every live instance by n_steps (one graph launch). Asynchronous.
 * n_steps == 0 only sorts in admitted instances, compacts retired ones and
 * builds the step graph for the current variant if it is not built yet
 * (otherwise the first stepping call pays that, about half a second). */
int tdem_batch_step(tdem_batch* h, int64_t n_steps, void* stream);

/* Integer-time state of one instance in its local order (host FP64 outputs,
 * any may be NULL) and its ledger (TDEM_BATCH_L_COUNT doubles). Runs one
 * read-back evaluation of that instance only. Synchronizes `stream`. */
int tdem_batch_read(tdem_batch* h, int32_t id, double* pos, double* vel, double* omega, double* force,
                    double* torque, double* ledger, int32_t ledger_count, void* stream);

/* Ledgers of `count` live instances (count x TDEM_BATCH_L_COUNT doubles,
 * host) from one read-back evaluation of all of them. Synchronizes `stream`. */
int tdem_batch_read_ledgers(tdem_batch* h, const int32_t* ids, int32_t count, double* out, void* stream);

/* Step limit of an instance (0: none): once it has taken `steps` steps it is
 * frozen (state carried over unchanged, no forces, no ledger) until it is
 * read and retired. Lets a serving loop run fixed-length step blocks while
 * instances finish at their own step counts. */
int tdem_batch_set_steps(tdem_batch* h, int32_t id, int64_t steps, void* stream);

/* Retire an instance: it stops at once; its particles, slot and key range
 * are reclaimed by the compaction rebuild at the next step boundary. */
int tdem_batch_retire(tdem_batch* h, int32_t id, void* stream);

/* Bond states of one instance: (lo, hi) local ids, (mode: 0 intact, 1
 * tensile, 2 shear, 3 both; instance evaluation of the break or -1). */
int tdem_batch_read_bonds(tdem_batch* h, int32_t id, int32_t* pairs, int32_t* state, int64_t capacity,
                          int64_t* count, void* stream);

/* Batch counters (TDEM_BATCH_I_COUNT int64). Synchronizes `stream`. */
int tdem_batch_info(tdem_batch* h, int64_t* out, int32_t count, void* stream);

/* Step-kernel variants (block shape, CTAs per SM, tiles per grab of the
 * work counter) and the autotuner that times `steps` real steps of each and
 * keeps the fastest. */
int tdem_batch_num_variants(void);
int tdem_batch_set_variant(tdem_batch* h, int variant);
int tdem_batch_get_variant(const tdem_batch* h);
int tdem_batch_autotune(tdem_batch* h, int steps, float* ms_out, void* stream);
int tdem_batch_use_graph(tdem_batch* h, int on);
int tdem_batch_last_error(const tdem_batch* h, char* buf, size_t len);

/* ========================================================================
 * 4. 3-D reference mode ("icedem3d"): the reference's IceDEM3D
 * ====================================================================== */

/* FP64 step of the reference's bonded-sphere engine
 * (src/tensordem/dem3d.py:564-1663): central-force bonds of the cubic
 * lattice (linear or Maxwell-Wiechert), tensile / objective-shear / creep
 * breakage, cell-list sphere contacts (linear penalty or Hertz, restitution
 * or absolute dashpot, Cundall-Strack friction with a pair-keyed history that
 * is never dropped, rolling-resistance couple), a spherical indenter, top /
 * bottom / lateral plane platens (with Coulomb friction), gravity, buoyancy,
 * wet drag and semi-implicit Euler. One CTA runs one instance for many steps
 * per launch; each particle's force is summed in the reference's index_add_
 * order. Derived constants are computed by the caller exactly as the
 * reference computes them (Python floats), so the kernel sees the same bits. */
typedef struct tdem_icedem3d tdem_icedem3d;

enum { TDEM_ICE3D_MAX_BRANCHES = 4 };

/* Friction-cone laws (DEM3DConfig.friction_cone_limit, dem3d.py:453-498). */
enum {
  TDEM_CONE_OFF = 0,   /* no tangential spring */
  TDEM_CONE_SINGLE,    /* limit = c0 N */
  TDEM_CONE_TANH,      /* limit = (c0 + c1 (1 - tanh(|v_t| / c2)) / 2) N */
  TDEM_CONE_DUAL       /* limit = |F_t| > c0 N ? c1 N : c0 N */
};

typedef struct {
  int32_t n;                 /* particles, 2 <= n <= tdem_icedem3d_max_particles() */
  int32_t nbond;             /* bonds (pairs i < j sorted by i * n + j) */
  int32_t hertz;             /* 0: linear penalty k_n; 1: Hertz (contact_model="hertz") */
  int32_t damping;           /* 0 none, 1 restitution-derived, 2 absolute (contact_damping) */
  int32_t hertz_tangential;  /* 1: k_t = hertz_kt sqrt(overlap); 0: constant tangential_k */
  int32_t rolling;           /* rolling-resistance couple on */
  int32_t platens;           /* bit0 top, bit1 bottom, bit2 lateral */
  int32_t body;              /* bit0 body forces on, bit1 water present, bit2 wet drag */
  int32_t n_branches;        /* Maxwell branches (0: linear bond) */
  int32_t creep;             /* Kachanov damage clock on */
  int32_t any_fixed;         /* some particle is fixed (pinned-pair effective mass) */
  double radius, mass, dt, drag;
  double bond_k;             /* linear k_b, or the equilibrium spring k0 */
  double branch_k[TDEM_ICE3D_MAX_BRANCHES];
  double branch_tau[TDEM_ICE3D_MAX_BRANCHES];
  double branch_decay[TDEM_ICE3D_MAX_BRANCHES];      /* exp(-dt / tau) */
  double branch_one_minus[TDEM_ICE3D_MAX_BRANCHES];  /* -expm1(-dt / tau) */
  double breaking_strain, shear_breaking_strain;
  double creep_exponent, creep_dt_over_time;         /* m, dt / t_ref */
  double contact_k;          /* linear penalty stiffness */
  double hertz_kn;           /* (4/3) E* sqrt(R*), particle pair */
  double hertz_kn_rigid;     /* (4/3) E* sqrt(R*), rigid counterpart */
  double hertz_pot;          /* (8/15) E* sqrt(R*), particle pair (contact energy) */
  double tangential_k, hertz_kt;
  double damping_c;          /* absolute: contact_damping; restitution, Hertz: 2 zeta */
  double gamma_mobile, gamma_pinned; /* restitution, linear: 2 zeta sqrt(k_n m_eff) */
  double mass_mobile, mass_pinned;   /* m / 2 and m */
  int32_t cone, platen_cone;         /* TDEM_CONE_* of particle and platen friction */
  double cone_c[3], platen_cone_c[3];
  double roll_mu;
  double tool_radius, tool_damping;
  double tool_start[3], tool_velocity[3];
  double platen_k, platen_c, platen_kt;
  double top_start_z, top_velocity, bottom_start_z, bottom_velocity;
  double lateral_k, lateral_c;
  double gravity_force;      /* m g */
  double buoyancy_force;     /* rho_w g (4/3) pi r^3 */
  double wet_drag;           /* C_wet */
  double water_level;
  double cap_denominator;    /* 4 r**3, the spherical-cap volume fraction's denominator */
  int32_t mindlin;           /* 1: Mindlin-Deresiewicz partial slip replaces the Cundall-Strack cone
                                (mindlin_partial_slip.py:174-232), for pairs and platens */
  int32_t pad3;
  double mindlin_platen_8g;  /* 8 G*, rigid counterpart (platen no-slip stiffness 8 G* a) */
  double rigid_radius;       /* R*, rigid counterpart */
  double rigid_4e;           /* 4 E*, rigid counterpart (contact radius a = (3 F R* / (4 E*))^(1/3)) */
} tdem_icedem3d_config;

/* Constant topology, host arrays, copied at create time. */
typedef struct {
  const int32_t* bond_i;       /* (B) */
  const int32_t* bond_j;       /* (B) */
  const double* rest_length;   /* (B) */
  const double* reference;     /* (B,3) x0[j] - x0[i] */
  const double* initial_normal;/* (B,3) */
  const double* threshold;     /* (B) per-bond tensile threshold, or NULL */
  const double* creep_reference; /* (B) Kachanov reference force, or NULL */
  const double* pinv;          /* (n,3,3) pseudo-inverse of each particle's bond covariance */
  const uint8_t* full_rank;    /* (n) covariance of rank 3 */
} tdem_icedem3d_topology;

/* Caller-owned state, device pointers, passed on every call. */
typedef struct {
  double* positions;           /* (n,3) */
  double* velocities;          /* (n,3) */
  const double* initial_positions; /* (n,3) */
  const uint8_t* fixed;        /* (n) */
  uint8_t* alive;              /* (B) */
  uint8_t* failure_mode;       /* (B) 1 tensile, 2 shear, 3 both, 4 creep */
  double* failure_time_s;      /* (B) */
  double* failure_extension_m; /* (B) */
  double* failure_energy_J;    /* (B) */
  double* branch_offsets;      /* (B, n_branches) or NULL */
  double* elongation_prev;     /* (B) or NULL */
  double* damage;              /* (B) or NULL */
  double* bond_dissipation;    /* (1) cumulative dashpot dissipation, or NULL */
  double* top_tangential;      /* (n,3) top platen spring offsets, or NULL */
  double* bottom_tangential;   /* (n,3) */
  double* lateral_position;    /* (4) x_min, x_max, y_min, y_max planes, or NULL */
  const double* lateral_velocity; /* (4) */
} tdem_icedem3d_state;

enum {
  TDEM_L3_REACTION_X = 0, TDEM_L3_REACTION_Y, TDEM_L3_REACTION_Z,
  TDEM_L3_TOP_REACTION_Z, TDEM_L3_BOTTOM_REACTION_Z,
  TDEM_L3_LATERAL_0, TDEM_L3_LATERAL_1, TDEM_L3_LATERAL_2, TDEM_L3_LATERAL_3,
  TDEM_L3_FRICTION_POWER, TDEM_L3_ROLLING_POWER,
  TDEM_L3_CONTACT_ENERGY,     /* contact potential of the evaluated configuration */
  TDEM_L3_CONTACTS,           /* overlapping pairs of the last evaluation */
  TDEM_L3_HISTORY_MAX,        /* largest friction-history table of a particle */
  TDEM_L3_STEPS_DONE, TDEM_L3_STATUS,
  TDEM_L3_MIN_BREAK_MARGIN,
  TDEM_L3_COUNT = 20
};

int tdem_icedem3d_max_particles(void);
int tdem_icedem3d_create(const tdem_icedem3d_config* cfg, const tdem_icedem3d_topology* topo,
                         tdem_icedem3d** out);
void tdem_icedem3d_destroy(tdem_icedem3d* h);

/* One force evaluation at `time` (IceDEM3D.forces, dem3d.py:1301-1642):
 * update_fracture commits breaks, update_history advances the friction and
 * Maxwell histories. Writes the total force (n,3) to `out_force` (device).
 * `loads`: optional (n,3) device array. */
int tdem_icedem3d_forces(tdem_icedem3d* h, const tdem_icedem3d_state* st, const double* loads,
                         double time, int update_fracture, int update_history, double* out_force,
                         void* stream);

/* `n_steps` steps from `time` (IceDEM3D.step, dem3d.py:1644-1663), loads held
 * over all of them. Synchronizes `stream`; TDEM_ERR_NONFINITE after the step
 * whose state stopped being finite, TDEM_ERR_CAPACITY when a contact list or
 * friction history of a particle overflowed. */
int tdem_icedem3d_step(tdem_icedem3d* h, const tdem_icedem3d_state* st, const double* loads,
                       int64_t n_steps, double time, void* stream);

/* How threads map onto particles (results are bitwise the same either way):
 * several lanes per particle (each owning whole sums), one thread per particle,
 * or by size (lanes while a 16-lane group fits every particle; the default). */
enum { TDEM_ICE3D_MAP_AUTO = 0, TDEM_ICE3D_MAP_LANES = 1, TDEM_ICE3D_MAP_PARTICLE = 2 };
int tdem_icedem3d_set_mapping(tdem_icedem3d* h, int mapping);
/* Naps of 64 ns a grid barrier of the cooperative step may wait before the
 * block records a timeout and returns (default 2^24, about a second). For
 * tests of the failure path: a short limit makes the barriers run out; the
 * launch then fails with TDEM_ERR_CUDA ("grid barrier timed out") and the
 * next launch starts clean. No counterpart in the reference. */
int tdem_icedem3d_set_barrier_spins(tdem_icedem3d* h, uint64_t spins);

/* Ledger of the last call (TDEM_L3_COUNT doubles). Synchronizes `stream`. */
int tdem_icedem3d_read_ledger(tdem_icedem3d* h, double* out_host, int count, void* stream);

/* Overlapping pairs (i < j) of the last evaluation, host int32 (count, 2). */
int tdem_icedem3d_read_contacts(tdem_icedem3d* h, int32_t* pairs_host, int64_t capacity, int64_t* count,
                                void* stream);
/* The pair friction history (the reference's IceDEM3D._tangential_state,
 * dem3d.py:1152-1185): `count` entries of pair (i < j, host int32 (count,2))
 * and stored tangential displacement (host double (count,3)). Set replaces
 * the whole table; read returns it in (i, then insertion) order. */
int tdem_icedem3d_set_history(tdem_icedem3d* h, const int32_t* pairs_host, const double* disp_host, int64_t count,
                              void* stream);
int tdem_icedem3d_read_history(tdem_icedem3d* h, int32_t* pairs_host, double* disp_host, int64_t capacity,
                               int64_t* count, void* stream);
int tdem_icedem3d_last_error(const tdem_icedem3d* h, char* buf, size_t len);

/* Host-side: the damping ratio zeta whose Hertz + Tsuji dashpot delivers the
 * requested restitution (contact_damping_model="restitution_calibrated";
 * replaces contact_calibration.hertz_damping_ratio_for_restitution,
 * src/tensordem/contact_calibration.py:219-248). No GPU needed. */
int tdem_hertz_damping_ratio(double restitution, double* zeta_out);

#ifdef __cplusplus
}
#endif

#endif /* TDEM_H_ */
