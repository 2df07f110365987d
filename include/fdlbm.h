/*
 * fdlbm - C ABI of the GB300 (sm_103a) two-phase D2Q9 lattice-Boltzmann step.
 *
 * The entry points replace, one for one, the step and boundary functions of
 * the reference scripts lattice_boltzmann/fingering_periodic.py (periodic in
 * y) and lattice_boltzmann/fingering.py (walls at bottom and top), plus
 * bounce_back.py.  Each declaration names the reference code it replaces.
 *
 * Conventions
 *   - All array arguments are DEVICE pointers unless stated otherwise; the
 *     caller owns every buffer (torch tensors, cudaMalloc, ...).
 *   - Populations are (9, H, W) direction-major, row-major planes; fields are
 *     (H, W) row-major; the element type is given by `dtype`.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous; errors detected on the host are returned immediately,
 *     launch errors are returned from the call that launched.
 *   - Every call returns FD_OK (0) or a negative FD_ERR_* code;
 *     fd_last_error() gives the message of the last failure on the calling
 *     host thread.
 *   - Macroscopic fields are stored on the full (H, W) grid; values on solid
 *     cells are not defined (the reference keeps them as 1-D arrays over fluid
 *     cells, fingering_periodic.py:103-113).
 */
#ifndef FDLBM_H
#define FDLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDLBM_ABI_VERSION 5

enum fd_status {
  FD_OK = 0,
  FD_ERR_ARG = -1,      /* null pointer, bad enum, bad size */
  FD_ERR_SHAPE = -2,    /* lattice shape not supported by this entry point */
  FD_ERR_CUDA = -3,     /* CUDA launch or runtime error */
  FD_ERR_DTYPE = -4,    /* dtype not supported by this entry point */
  FD_ERR_SCRATCH = -5,  /* request larger than a fixed scratch area */
  FD_ERR_NONFINITE = -6 /* a step met a non-finite density or psi (the reference raises
                           FloatingPointError there, np.seterr(all='raise'), fingering_periodic.py:496) */
};

/* Bits of the device status word (fd_device_status). */
#define FD_STATUS_WAIT_TIMEOUT 1u /* a bounded wait on an asynchronous copy gave up */
#define FD_STATUS_NONFINITE 2u    /* a packed fused step (fd_fused_step_packed, _host, _noalloc) met a
                                     fluid cell whose density or psi is not finite */

enum fd_dtype { FD_F64 = 0, FD_F32 = 1, FD_F16 = 2, FD_BF16 = 3 };

enum fd_variant {
  FD_VARIANT_PERIODIC = 0, /* fingering_periodic.py: y periodic, Gaussian inlet, outlet 2/3 */
  FD_VARIANT_WALLS = 1,    /* fingering.py: psi_wall ghost rows, walls on rows 1 and H-2, corners, outlet 1.5 */
  FD_VARIANT_PERIODIC_XY = 2 /* extension, no reference counterpart: periodic in x and y (no Zou-He, no x ghost
                                columns) with the body force (force_x, force_y) per unit mass on both fluids;
                                FP64 / FP32 reference-order kernels only */
};

/* fd_params.flags */
#define FD_INIT_MU 1u /* Compute.__init__ evaluates mu before the equilibria (fingering.py:122) */
#define FD_INIT_UY 2u /* ... and u_y with f = 0 (fingering.py:123) */
#define FD_OUTLET_PRESSURE 8u /* extension, no reference counterpart: Zou-He pressure outlet rho = 1 at x = W-1
                                 (u_x from the known populations, coefficient 2/3) instead of the reference's
                                 velocity-type outlet; both variants, every kernel */
#define FD_INIT_VELOCITY 4u /* fd_compute_init takes u_x, u_y from the fields' ux / uy arrays (the
                               equilibrium of a given flow: restarting from predicted fields; no
                               counterpart in the reference, whose runs start at rest) */

/* Model constants, the reference's module globals (fingering_periodic.py:15-44). */
typedef struct fd_params {
  int32_t H, W;
  int32_t variant;     /* enum fd_variant */
  uint32_t flags;      /* FD_INIT_* */
  double tau;          /* g relaxation time */
  double eta_n;        /* Eta_n */
  double M;            /* viscosity ratio */
  double a, kappa;     /* free-energy coefficients */
  double gamma;        /* mobility */
  double psi_wall;     /* psi on solid cells */
  double outlet_coef;  /* 2/3 (fingering_periodic.py:317) or 1.5 (fingering.py:378) */
  double force_x;      /* FD_VARIANT_PERIODIC_XY: body force per unit mass (Guo forcing, as mu grad psi) */
  double force_y;
} fd_params;

/* Device pointers of the reference's Compute attributes (fingering_periodic.py:90-121). */
typedef struct fd_fields {
  void* f;        /* (9,H,W) */
  void* g;        /* (9,H,W) */
  void* psi;      /* (H,W) order parameter, psi_wall on solid */
  void* npx;      /* (H,W) nabla_psix */
  void* npy;      /* (H,W) nabla_psiy */
  void* np2;      /* (H,W) nabla_psi2 */
  void* rho;      /* (H,W) */
  void* ux;       /* (H,W) */
  void* uy;       /* (H,W) */
  void* p;        /* (H,W) */
  void* mu;       /* (H,W) */
  void* mix_tau;  /* (H,W) */
} fd_fields;

/* Selector of fd_collision_term (fingering_periodic.py:194-199, 171-192, 258-264). */
enum fd_term { FD_TERM_LARGE_F = 0, FD_TERM_FEQ = 1, FD_TERM_GEQ = 2, FD_TERM_F = 3, FD_TERM_G = 4 };

/* Selector of fd_field (fingering_periodic.py:123-256). */
enum fd_field_id {
  FD_FIELD_RHO = 0,      /* getRho       fingering_periodic.py:151 */
  FD_FIELD_NPX = 1,      /* getNabla_psix fingering_periodic.py:214 */
  FD_FIELD_NPY = 2,      /* getNabla_psiy fingering_periodic.py:228 */
  FD_FIELD_NP2 = 3,      /* getNabla_psi2 fingering_periodic.py:242 */
  FD_FIELD_MU = 4,       /* getMu        fingering_periodic.py:141 */
  FD_FIELD_MU_PLAIN = 5, /* getMu_plain  fingering_periodic.py:146 */
  FD_FIELD_UX = 6,       /* getUx        fingering_periodic.py:126 */
  FD_FIELD_UY = 7,       /* getUy        fingering_periodic.py:134 */
  FD_FIELD_P = 8,        /* getP         fingering_periodic.py:123 */
  FD_FIELD_MIX_TAU = 9,  /* getMix_tau   fingering_periodic.py:201 */
  FD_FIELD_PSI = 10      /* udpatePsi    fingering_periodic.py:210 (sum of g, psi_wall on solid) */
};

/* ---- library ------------------------------------------------------------ */
int fd_abi_version(void);
const char* fd_last_error(void);

/* ---- reference-order step, one entry per reference function (FP64 / FP32) -- */

/* Compute.__init__ (fingering_periodic.py:48-121; fingering.py:54-127).
 * psi0: (H,W) double initial psi before solid cells are set to psi_wall;
 * rho0: (H,W) double initial density or NULL for 1.0.  Writes every member of
 * `out`; populations on solid cells are zero. */
int fd_compute_init(const fd_params* prm, int dtype, const uint16_t* mask, const double* psi0,
                    const double* rho0, const fd_fields* out, void* stream);

/* Regularised restart (no counterpart in the reference, whose runs start at
 * rest): adds to populations that hold the equilibrium of given fields (as
 * fd_compute_init with FD_INIT_VELOCITY writes them) the first-order
 * non-equilibrium part of that flow, f_i += -3 w_i tau_mix Q_i : S(rho u) and
 * g_i += -3 w_i tau Q_i : S(psi u), Q_i = e_i e_i - I/3, S the symmetric
 * velocity-flux gradient by central differences over fluid neighbours.  Density,
 * psi and momentum are unchanged.  Fluid cells only; `fields` holds rho, psi,
 * ux, uy and mix_tau of the state (as fd_compute_init leaves them). */
int fd_add_nonequilibrium(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields,
                          void* stream);

/* The collision loop body for all nine directions, fluid cells only:
 * f[j][mask] = getF(j), g[j][mask] = getG(j) with F, feq, geq from the stored
 * fields (fingering_periodic.py:455-460). In place on fields->f, fields->g. */
int fd_collide(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields, void* stream);

/* One of getLarge_F(j), getfeq(j), getgeq(j), getF(j), getG(j)
 * (fingering_periodic.py:194-199, 171-181, 183-192, 258-260, 262-264) on the
 * full grid; `out` is (H,W) and is written on fluid cells only. */
int fd_collision_term(const fd_params* prm, int dtype, int term, int j, const uint16_t* mask,
                      const fd_fields* fields, void* out, void* stream);

/* stream(f, g) (fingering_periodic.py:327-343): dst = src shifted by e_i,
 * periodic in x and y, every cell.  src and dst must not overlap. */
int fd_stream(const fd_params* prm, int dtype, const void* src_f, const void* src_g, void* dst_f,
              void* dst_g, void* stream);

/* Bounce_back.halfway_bounceback_rec / halfway_bounceback_circle
 * (bounce_back.py:25-86, 89-167) and the wall rows of bottom_top_wall as
 * called by fingering.py:573, expressed as link bits of `mask`:
 * f_i(x) = f_behind_opp(i)(x) wherever bit i-1 of mask(x) is set. */
int fd_bounce_back(const fd_params* prm, int dtype, const uint16_t* mask, const void* f_behind,
                   const void* g_behind, void* f, void* g, void* stream);

/* bottom_top_wall(f_behind, g_behind, f, g) (fingering.py:432-451) on
 * arbitrary (9, rows, cols) views: row 0 of the view takes populations
 * 2,5,6 from 4,7,8 of f_behind, row rows-1 takes 4,7,8 from 2,5,6.
 * Strides are in elements. */
int fd_bottom_top_wall(int dtype, int rows, int cols, ptrdiff_t plane_stride, ptrdiff_t row_stride,
                       const void* f_behind, const void* g_behind, void* f, void* g, void* stream);

/* The psi_x, psi_y, mu_plain values zou_he_boundary_inlet/outlet recompute
 * from the stored psi and nabla_psi2 (fingering_periodic.py:273-275, 309-311),
 * at columns 0 and W-1: side = 6 x H values of dtype
 * [gx0, gy0, mu0, gxW, gyW, muW]. */
int fd_boundary_fields(const fd_params* prm, int dtype, const uint16_t* mask, const void* psi,
                       const void* np2, void* side, void* stream);

/* zou_he_boundary_inlet (fingering_periodic.py:268-302; fingering.py:298-364).
 * inlet_ux: (H) double u_x per row. */
int fd_zou_he_inlet(const fd_params* prm, int dtype, void* f, void* g, const void* side,
                    const double* inlet_ux, void* stream);

/* zou_he_boundary_outlet (fingering_periodic.py:305-324; fingering.py:369-390). */
int fd_zou_he_outlet(const fd_params* prm, int dtype, void* f, void* g, const void* side,
                     const double* inlet_ux, void* stream);

/* udpatePsi (fingering_periodic.py:210-212) into fields->psi, and
 * getRho (fingering_periodic.py:151-152) into fields->rho. */
int fd_update_rho_psi(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields,
                      void* stream);

/* The macroscopic tail of the loop body (fingering_periodic.py:472-479):
 * nabla_psix/psiy/psi2 from psi, then mu, ux, uy, p, mix_tau on fluid cells. */
int fd_update_macros(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields,
                     void* stream);

/* One getter of fingering_periodic.py:123-256 evaluated from the stored
 * fields into `out` ((H,W)). */
int fd_field(const fd_params* prm, int dtype, int field_id, const uint16_t* mask, const fd_fields* fields,
             void* out, void* stream);

/* ---- fused step --------------------------------------------------------- */

/* `nsteps` iterations of the main loop body (fingering_periodic.py:454-479,
 * fingering.py:558-585) as one kernel per iteration.  The state between
 * kernels is the post-collision population pair; the kernel pulls it
 * (stream + bounce-back + walls + Zou-He of iteration n-1), forms psi, its
 * stencils and the macroscopic fields of iteration n, and collides.
 *   pop_a, pop_b : two buffers of 18*H*W elements (f planes then g planes);
 *                  the state starts in pop_a and ping-pongs; after the call
 *                  it is in pop_a if nsteps is even, else in pop_b.
 *   side_a, side_b: two 6*H buffers of boundary fields; the values of the
 *                  state's iteration start in side_a and follow the same
 *                  ping-pong.
 * dtype: FD_F64 or FD_F32 (the storage and compute type).  W must be a
 * multiple of 4 and H >= 3.  rows_per_warp: rows one warp marches (0 = auto). */
int fd_fused_step(const fd_params* prm, int dtype, const uint16_t* mask, const double* inlet_ux,
                  void* pop_a, void* pop_b, void* side_a, void* side_b, int nsteps, int rows_per_warp,
                  void* stream);

/* ---- fused step with packed (deviation) storage --------------------------- */

/* Storage of the packed population buffers.  The f populations are stored as
 * deviations (f_i - w_i) * 2^f_scale_log2 and g_1..g_8 as g_i * 2^g_scale_log2
 * in `dtype` (FD_F32, FD_F16 or FD_BF16); g_0, which carries most of psi, is
 * always FP32.  Arithmetic is FP32 in every case.  The layout is 18 planes of
 * H*W elements, each starting on a 256-byte boundary: f_0..f_8, g_0, g_1..g_8.
 * There is no counterpart in the reference (it stores float64 only).
 *
 * Rounding of the FP16/BF16 stores of the fused step: FD_ROUND_NEAREST
 * (round to nearest even) or FD_ROUND_STOCHASTIC (round up with probability
 * equal to the discarded fraction, from a counter-based hash of the cell index
 * and the step's seed).  Round-to-nearest makes the same error in every cell
 * of a uniform region at every step, so the error accumulates as a drift of
 * the colour masses; stochastic rounding makes it zero-mean.  Step s of a call
 * (s = 0 .. nsteps-1) uses seed + s; results are reproducible for a given
 * seed.  pack/unpack always round to nearest; FD_F32 ignores both fields. */
enum fd_rounding { FD_ROUND_NEAREST = 0, FD_ROUND_STOCHASTIC = 1 };

typedef struct fd_storage {
  int32_t dtype;
  int32_t f_scale_log2;
  int32_t g_scale_log2;
  int32_t rounding;   /* fd_rounding */
  uint32_t seed;      /* stochastic rounding: seed of the first step of a call */
} fd_storage;

/* Bytes of one packed population buffer (0 on invalid arguments). */
size_t fd_packed_bytes(int H, int W, const fd_storage* st);

/* Reference-layout populations (18 planes of src_dtype: f then g) -> packed. */
int fd_pack(const fd_params* prm, int src_dtype, const void* src, const fd_storage* st, void* dst, void* stream);

/* Packed -> reference layout (18 planes of dst_dtype). */
int fd_unpack(const fd_params* prm, const fd_storage* st, const void* src, int dst_dtype, void* dst, void* stream);

/* fd_fused_step on packed buffers (the same loop body, fingering_periodic.py:454-479
 * / fingering.py:558-585, computed in FP32 in deviation form).  pop_a/pop_b:
 * fd_packed_bytes() each, 256-byte aligned; side_a/side_b: 6*H floats.
 * W must be a multiple of 4.  rows_per_warp: for W a multiple of 8 the strip
 * height in rows of the staged kernel (one CTA per band of 128 cells and strip),
 * otherwise the rows one warp of the register kernel marches; 0 = automatic. */
int fd_fused_step_packed(const fd_params* prm, const fd_storage* st, const uint16_t* mask, const double* inlet_ux,
                         void* pop_a, void* pop_b, void* side_a, void* side_b, int nsteps, int rows_per_warp,
                         void* stream);

/* fd_fused_step_packed for callers that cannot allocate device memory: a
 * host whose memory manager owns all of device memory (a framework's caching
 * allocator, or an arena reserved at start-up) and does not let a library call
 * cudaMalloc behind its back.  The caller passes its state only: pop_a / pop_b
 * as in fd_fused_step_packed and ONE boundary buffer `side` (6*H floats, the
 * state's boundary values on entry and on return).  The second boundary buffer
 * is a fixed 384 KiB array inside this library (6 x 16384 floats), held on
 * every GPU that loads the library until the process exits; H > 16384 is
 * rejected with FD_ERR_SCRATCH.  The call allocates nothing (no cudaMalloc, no
 * cudaFree, no allocating library routine).  Set-up on the first call on a
 * device (and again after the device's context was torn down and created
 * anew): the array's device address is looked up; the first call with a given
 * storage type and rounding also raises the chosen kernel's shared-memory
 * limit, as fd_fused_step_packed does, so make that first call before any
 * stream capture.  All calls share the array, so calls that overlap on the GPU
 * (other streams, other host threads) race; nothing in it needs clearing,
 * every iteration writes all of it before it is read.  No counterpart in the
 * reference. */
int fd_fused_step_packed_noalloc(const fd_params* prm, const fd_storage* st, const uint16_t* mask,
                                 const double* inlet_ux, void* pop_a, void* pop_b, void* side, int nsteps,
                                 int rows_per_warp, void* stream);

/* The step for a caller whose state lives in HOST memory, as the reference's
 * numpy arrays do (its loop body, fingering_periodic.py:454-479 /
 * fingering.py:558-585, on arrays it owns): the packed state in `host_in`
 * (fd_packed_bytes(), the device layout) is uploaded into pop_a, advanced
 * nsteps (>= 1) iterations as fd_fused_step_packed would (same results bit for
 * bit, same seeds), and the result is downloaded into `host_out`.  side_a
 * holds the boundary values of the state on entry (device, 6*H floats, as for
 * fd_fused_step_packed); the device state after the call is in pop_b / side_b
 * when nsteps is odd, else in pop_a / side_a.  The upload, the first and last
 * iterations and the download are pipelined over chunks of about chunk_rows
 * rows (<= 0: about 1/16 of the lattice; rounded to whole strips of 16 rows,
 * after four smaller leading chunks): both copy directions run at once and
 * the kernels run under them.  host_in may equal
 * host_out.  Host buffers should be pinned (cudaHostAlloc / cudaHostRegister),
 * or the copies do not overlap.  W must be a multiple of 8.  Asynchronous on
 * `stream` like every step; uses two internal streams per device, and calls on
 * one device from several host threads serialise while they enqueue.  No
 * counterpart in the reference (its state never leaves host memory). */
int fd_fused_step_packed_host(const fd_params* prm, const fd_storage* st, const uint16_t* mask,
                              const double* inlet_ux, const void* host_in, void* host_out, void* pop_a,
                              void* pop_b, void* side_a, void* side_b, int nsteps, int chunk_rows, void* stream);

/* ---- batched ensemble ----------------------------------------------------- */

/* One member of a batch: its parameters and its packed buffers (as for
 * fd_fused_step_packed).  No counterpart in the reference, which runs one
 * lattice per process. */
typedef struct fd_instance {
  fd_params prm;
  const uint16_t* mask;     /* device, H*W */
  const double* inlet_ux;   /* device, H */
  void* pop_a;              /* device, fd_packed_bytes(): the state at parity 0 */
  void* pop_b;
  void* side_a;             /* device, 6*H floats: the state's boundary values at parity 0 */
  void* side_b;
  uint32_t seed;            /* stochastic rounding: seed of the batch's first step for this member;
                               batch step k uses seed + k, as fd_fused_step_packed would */
} fd_instance;

typedef struct fd_batch fd_batch;

/* Build a batch over n members sharing one packed storage type (unscaled).
 * Every iteration is one persistent launch of the staged kernel over a table
 * of (member, band, strip) tiles: bands of band_width cells (64, 128, 256) and
 * strips of at most rows_per_strip rows (a member's strips are of equal
 * height within one row).  Allocates the (small) device tables. */
int fd_batch_create(const fd_instance* inst, int n, const fd_storage* st, int rows_per_strip, int band_width,
                    fd_batch** out);

/* Change the tile shape (drops a captured graph).  The new tile table leaves
 * out the members flagged non-finite (fd_batch_member_status), which the
 * batch no longer steps, so that the live members' tiles share the persistent
 * grid; a member whose flag was cleared is taken back by the next call. */
int fd_batch_configure(fd_batch* b, int rows_per_strip, int band_width);

/* Advance every member nsteps iterations on `stream`.  use_graph != 0 replays
 * a captured two-iteration CUDA graph (needs a non-default stream; the graph
 * is captured on first use). */
int fd_batch_step(fd_batch* b, int nsteps, int use_graph, void* stream);

/* 0 if the members' states are in pop_a / side_a, 1 if in pop_b / side_b. */
int fd_batch_parity(const fd_batch* b);

/* Quarantine of diverging members.  Every launch checks each fluid cell's
 * density and psi; a member with a non-finite one is flagged (out[i] != 0) and
 * its tiles are skipped by every later launch (its state stays as it was
 * then), while the other members keep stepping.  The reference aborts the whole
 * run instead (np.seterr(all='raise'), fingering_periodic.py:496).  Copies the
 * n member flags to the HOST array `out` after waiting for the device; clear
 * != 0 then releases every member (after the caller has restored its state).
 * Returns FD_ERR_NONFINITE if any member is flagged, FD_OK otherwise. */
int fd_batch_member_status(fd_batch* b, uint32_t* out, int clear);

/* Number of tiles per iteration. */
int fd_batch_tiles(const fd_batch* b);

/* CTAs of the persistent launch (resident CTAs per SM x SMs, at most the tile
 * count).  The CTAs take tiles from a counter, tallest strips first; a tile
 * count just under a whole number of rounds of the grid avoids a last round in
 * which a few CTAs run while the rest wait. */
int fd_batch_grid(const fd_batch* b);

int fd_batch_destroy(fd_batch* b);

/* ---- diagnostics -------------------------------------------------------- */

/* FP64 diagnostics of a state (no counterpart in the reference, which only
 * plots psi; defined here as the quantities an invasion is judged by). */
typedef struct fd_diag {
  double mass_r;        /* sum over fluid cells of rho (1 + psi) / 2 (invading fluid) */
  double mass_b;        /* sum over fluid cells of rho (1 - psi) / 2 (defending fluid) */
  double saturation;    /* invaded / fluid */
  int64_t invaded;      /* fluid cells with psi > 0 */
  int64_t fluid;        /* fluid cells */
  int32_t tip_x;        /* largest x of a fluid cell with psi > 0, -1 if none */
  int32_t breakthrough; /* 1 if a fluid cell with x >= W-5 has psi > 0 (the outlet rule pins
                           psi = -1 on column W-1 itself) */
} fd_diag;

/* Bytes of the scratch buffer fd_diagnostics needs (independent of the size). */
size_t fd_diag_scratch_bytes(void);

/* Diagnostics of a state held as reference-layout populations (st == NULL,
 * dtype FD_F64 / FD_F32, 18 planes) or as a packed buffer (st != NULL).
 * rho = sum f, psi = sum g per cell (the collision conserves both, so pre- and
 * post-collision states agree).  `out` is a DEVICE fd_diag; accumulation is in
 * FP64 in a fixed order, so results are reproducible. */
int fd_diagnostics(const fd_params* prm, int dtype, const fd_storage* st, const void* pop, const uint16_t* mask,
                   void* scratch, fd_diag* out, void* stream);

/* Self-test of the failure path: one thread waits, through the staged kernel's
 * bounded mbarrier wait, on a barrier that nothing arrives on; after `polls`
 * polls (1 .. 2^20) the wait gives up and bit 0 of the device error word is set
 * (read with fd_device_status).  unit 0 runs it in the code unit of the
 * single-lattice kernels, unit 1 in that of the batched kernel (each unit of
 * the library has its own copy of the word).  Faults, traps and hangs nothing.
 * No counterpart in the reference. */
int fd_selftest_wait_timeout(unsigned polls, int unit, void* stream);

/* Device-side status word of the library's kernels (FD_STATUS_* bits: a
 * bounded wait on an asynchronous copy gave up; a packed fused step met a
 * non-finite density or psi), the OR over the library's code units.  Copies
 * it to *out and, if clear != 0, resets it.  Synchronous.  No counterpart in the reference (numpy raises
 * instead, fingering_periodic.py:497). */
int fd_device_status(unsigned* out, int clear);

#ifdef __cplusplus
}
#endif

#endif /* FDLBM_H */
