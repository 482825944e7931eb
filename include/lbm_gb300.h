/*
 * lbm_gb300.h -- C-ABI of liblbm_gb300.so, a GB300 (sm_103a) implementation of
 * the Zheng-Shu-Chew free-energy multiphase lattice Boltzmann step
 * (D3Q7 order-parameter distribution f + D3Q19 momentum distribution g).
 *
 * The reference (carlosrosales/lbm_bench_gpu) has no library boundary: its
 * driver src/main.cu allocates ~40 device arrays, copies constants with
 * cudaMemcpyToSymbol and launches thirteen kernels (seven compute, six
 * pack/unpack) plus three host-staged halo exchanges per step.  Each entry point below replaces one stage of that
 * driver; the citation next to it names the reference lines it stands for.
 *
 * Conventions
 *  - Names follow the reference: f = D3Q7 (phi, relaxed with tauPhi),
 *    g = D3Q19 (momentum, relaxed with tauRho), rho = ZSC mean density n.
 *  - Host arrays are caller-owned, x fastest: idx = x + nx*(y + ny*z), with
 *    z in [0, nz) standing for the reference's interior plane k = z + 1.
 *  - Every function returns an LBM_* status and never aborts.
 *  - One host thread per context.  lbm_step is asynchronous on the context's
 *    CUDA stream; every call that hands data back to the host synchronises.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LBM_OK 0
#define LBM_EINVAL 1      /* bad argument or unsupported size */
#define LBM_ENOMEM 2      /* device or host allocation failed */
#define LBM_ECUDA 3       /* a CUDA call or a kernel launch failed */
#define LBM_ENAN 4        /* the state holds NaN or Inf */
#define LBM_ETIMEOUT 5    /* a bounded device wait gave up */
#define LBM_EIO 6         /* an input file is missing or malformed */
#define LBM_ESTATE 7      /* call out of order (e.g. adjoint without a recorded forward) */

/* storage formats of the distributions (arithmetic is always FP32) */
#define LBM_STORAGE_FP32 0
#define LBM_STORAGE_FP16 1   /* shifted, scaled half precision */
#define LBM_STORAGE_BF16 2   /* shifted, scaled bfloat16 */

typedef struct lbm_ctx lbm_ctx;

/* The physical and numerical inputs of properties.in (src/paramread.c:40-59)
 * plus the radius of the first bubble of discrete.in, which sets the gravity
 * scale (src/paramread.c:160). */
typedef struct lbm_params {
    int nx, ny, nz;           /* xmax ymax zmax: interior nodes */
    int block_x, block_y;     /* BLOCK_SIZE_X BLOCK_SIZE_Y: validated in compat mode, not used for launch */
    float rhoL, rhoH;
    float tauRho, tauPhi;
    float width, sigma, Gamma;
    float Eo;
    float rc0;                /* Rc of the first bubble */
    int storage;              /* LBM_STORAGE_* */
    int device;               /* CUDA device ordinal */
    int compat;               /* 1: reject what src/main.cu:167-173 rejects */
} lbm_params;

/* The step counters of properties.in (src/paramread.c:41-42). */
typedef struct lbm_run {
    int max_step, relax_step, save, stat;
} lbm_run;

/* Derived constants, src/paramread.c:141-170 (computed in double, stored as float). */
typedef struct lbm_derived {
    float phiStar, phiStarSq;
    float invTauRho, invTauRhoOne, invTauRhoHalf;
    float eta, eta2, invEta2;
    float invTauPhi, invTauPhiOne;
    float alpha, alpha4, kappa;
    float gravity, grav;      /* grav: the body force of the evolution loop (src/main.cu:479) */
    float K0, K1, K2, KC0, KC1, KC2;
} lbm_derived;

/* Statistics over the phi, rho, u arrays.
 * "compat" values reproduce src/stats.c:39-91 and src/logsave.c:63-167: they
 * skip the planes x = 0, nx-1 and y = 0, ny-1, as the reference does, and
 * Pout divides by nx*ny*nz - vol.  The full-domain sums are FP64 over every
 * node. */
typedef struct lbm_stats_out {
    long long step;           /* steps taken since lbm_init */
    double umax;              /* compat: sqrt(max |u|^2) */
    double vol;               /* compat: number of nodes with phi >= 0 */
    double ux_av, uy_av, uz_av;   /* compat: mean u over phi >= 0 */
    double ref;               /* compat: (0.75 vol / pi)^(1/3) */
    double p_in, p_out, p_dif, p_err;   /* compat: Laplace-law check */
    double phi_sum, rho_sum;  /* full domain: sum phi, sum rho */
    double mom_x, mom_y, mom_z;         /* full domain: sum rho u */
    double vol_full;          /* full domain: number of nodes with phi >= 0 */
    double umax_full;         /* full domain: sqrt(max |u|^2) */
    long long nonfinite;      /* nodes whose phi, rho or u is NaN or Inf */
} lbm_stats_out;

/* Parse dir/properties.in and dir/discrete.in in the reference's positional
 * format (src/paramread.c:36-75; header tokens are skipped by count).
 * bubbles receives up to max_bubbles rows of {xc, yc, zc, Rc}; *nbubbles is
 * the count in the file.  dir NULL means the current directory. */
int lbm_read_inputs(const char *dir, lbm_params *p, lbm_run *run, float *bubbles, int max_bubbles,
                    int *nbubbles);

/* Derived constants for p (src/paramread.c:141-170). */
int lbm_derive(const lbm_params *p, lbm_derived *d);

/* Create a context and the initial state from host fields, each nx*ny*nz
 * values: host init -> upload -> init_f/init_g of src/main.cu:294-358.  The
 * initial equilibrium is at rest (src/init_f.cu:72-78, src/init_g.cu:77-91);
 * u0 only fills the velocity arrays.  phi_ghost may be NULL (periodic z) or
 * 2*nx*ny values: the plane below z = 0, then the plane above z = nz-1, which
 * the reference fills from the bubble geometry (src/init.c:41-59). */
int lbm_init(lbm_ctx **out, const lbm_params *p, const float *phi0, const float *rho0, const float *ux0,
             const float *uy0, const float *uz0, const float *phi_ghost);

/* As lbm_init, with the bubble initial condition computed on the GPU
 * (src/init.c:39-59: phi = -phiStar, then for each bubble in order, nodes with
 * R <= Rc + width take phiStar*tanh(2(Rc - R)/width); rho = (rhoH + rhoL)/2;
 * u = 0; ghost planes from the geometry).  bubbles: nbubbles rows of
 * {xc, yc, zc, Rc} in the reference's coordinates (x, y 0-based, z 1-based). */
int lbm_init_bubbles(lbm_ctx **out, const lbm_params *p, const float *bubbles, int nbubbles);

/* Advance nsteps time steps with body force grav (0 while relaxing): the loop
 * bodies of src/main.cu:363-473 and :496-608 without their stats/vtk output.
 * One fused kernel per step.  Asynchronous on the context's stream. */
int lbm_step(lbm_ctx *c, int nsteps, float grav);

/* Statistics (see lbm_stats_out) of the phi, rho, u arrays as the reference
 * holds them: the moments computed at the start of the last step
 * (src/update_phi.cu, src/update_rho.cu, src/update_velocity.cu), or the
 * initial fields before any step.  Replaces src/stats.c:28-96 and the pressure
 * part of src/logsave.c:63-167.  Each non-NULL field pointer receives
 * nx*ny*nz floats.  s may be NULL.  Returns LBM_ENAN (after filling s) when a
 * field holds NaN or Inf.  Synchronises. */
int lbm_stats(lbm_ctx *c, lbm_stats_out *s, float *phi, float *rho, float *ux, float *uy, float *uz);

/* The same statistics of caller-supplied host fields (nx*ny*nz floats each,
 * all required), reduced on the context's GPU.  The reference computes its
 * statistics and Laplace check on its host copies of the fields
 * (src/stats.c:28-96, src/logsave.c:63-167), which it refreshes only at its
 * output points (phi and u every `stat` steps, rho every `save` steps,
 * src/main.cu:457-472); a driver that keeps host copies on the same schedule
 * reproduces its logs exactly with this call.  Synchronises. */
int lbm_stats_fields(lbm_ctx *c, lbm_stats_out *s, const float *phi, const float *rho, const float *ux,
                     const float *uy, const float *uz);

/* Pressure of every node from the current phi and rho (the expression of
 * src/vtksave.c:63-127, periodic neighbours) into nx*ny*nz host floats.
 * Synchronises. */
int lbm_pressure(lbm_ctx *c, float *p);

/* Name (NUL-terminated, truncated to len - 1 characters) and total memory of
 * a CUDA device, for run logs (src/main.cu:94-119, src/logsave.c:189-194).  Either output may be
 * NULL. */
int lbm_device_name(int device, char *name, int len, double *total_bytes);

/* The current distributions in streamed form, as the reference's lower halves
 * hold them after a step: f as 7 blocks and g as 19 blocks of nx*ny*nz floats
 * (reference direction order).  NULL skips.  Synchronises. */
int lbm_get_dist(lbm_ctx *c, float *f, float *g);

/* Replace the state by streamed distributions (same layout as lbm_get_dist),
 * e.g. to resume from a snapshot.  The phi, rho, u arrays are recomputed as
 * their moments.  Synchronises. */
int lbm_set_dist(lbm_ctx *c, const float *f, const float *g);

/* Objectives of lbm_step_adjoint, on the moments of the streamed state
 * (phi = sum f, rho = sum g, u = sum c g / rho) with the smooth light-phase
 * weight w = (phiStar - phi) / (2 phiStar):
 *   LBM_OBJ_LIGHT_UZ_MEAN     mean over the last `window` states of
 *                             sum(w u_z) / sum(w): rise velocity of the light phase
 *   LBM_OBJ_LIGHT_Z_CENTROID  sum(w z) / sum(w) of the final state (z = plane
 *                             index + 1, the reference's z coordinate) */
#define LBM_OBJ_LIGHT_UZ_MEAN 0
#define LBM_OBJ_LIGHT_Z_CENTROID 1

typedef struct lbm_adjoint_opts {
    int objective;            /* LBM_OBJ_* */
    int nsteps;               /* T: steps of the run, starting from the initial state */
    int window;               /* states averaged by LBM_OBJ_LIGHT_UZ_MEAN (the last `window`) */
    float grav;               /* body force of the run */
    double checkpoint_bytes;  /* device memory for checkpoints; <= 0: the free memory less a reserve of
                                 max(4 GiB, 5% of the device) */
    double host_checkpoint_bytes;   /* pinned host memory for a second checkpoint tier (0: none): the
                                       states at the starts of equal segments go to the host during
                                       the first forward sweep, and each segment is reversed from its
                                       start with the device checkpoints */
} lbm_adjoint_opts;

typedef struct lbm_adjoint_out {
    double J;                 /* objective (FP64 accumulation) */
    double dJ_dgrav;          /* dJ / d grav (FP64 accumulation) */
    float *dJ_dphi0;          /* caller's nx*ny*nz host buffer for dJ / d phi0, or NULL */
    int slots;                /* checkpoints held, the initial state included */
    long long forward_steps;  /* forward steps run, recomputation included */
    long long adjoint_steps;  /* = nsteps */
    double seconds;           /* wall time of the call */
    double checkpoint_bytes_used;
    int host_slots;           /* segment starts held in host memory (0: one tier) */
} lbm_adjoint_out;

/* Gradient of an objective over T steps with respect to the body force and
 * the initial phi field, by the discrete adjoint of the fused step (reverse
 * streaming, transposed collisions, transposed gradient / Laplacian stencils,
 * force terms) with binomial checkpointing of the forward trajectory.  No
 * counterpart in the reference.  The context must hold its initial state
 * (lbm_init / lbm_init_bubbles / lbm_set_dist, no step taken); the gradient
 * with respect to phi0 passes through the initial equilibrium with periodic
 * z.  On return the context holds the initial state again.  Synchronises.
 * The work buffers and the checkpoint pool stay allocated in the context for
 * the next call (a pool larger than the next budget is reused, not shrunk)
 * until lbm_adjoint_release or lbm_destroy; checkpoint_bytes <= 0 counts the
 * cached pool as free memory. */
int lbm_step_adjoint(lbm_ctx *c, const lbm_adjoint_opts *o, lbm_adjoint_out *out);

/* The objective of lbm_step_adjoint alone (forward run, no gradient), e.g.
 * for finite-difference checks of the gradient: o->checkpoint_bytes is
 * ignored, one state snapshot is held.  No counterpart in the reference.
 * Same preconditions; on return the context holds the initial state again.
 * Synchronises. */
int lbm_objective(lbm_ctx *c, const lbm_adjoint_opts *o, double *J);

/* Free the adjoint work buffers and checkpoint pool that lbm_step_adjoint and
 * lbm_objective keep in the context.  No counterpart in the reference.
 * Synchronises the context's stream. */
int lbm_adjoint_release(lbm_ctx *c);

/* Forward steps lbm_step_adjoint runs for nsteps steps with `slots` device
 * checkpoint slots and `host_slots` host ones (host_checkpoint_bytes divided
 * by the snapshot bytes; 0: lbm_adjoint_forward_steps), without running it.
 * No counterpart in the reference.  -1 for bad arguments. */
long long lbm_adjoint_forward_steps_tiers(long long nsteps, int slots, long long host_slots);

/* Forward steps lbm_step_adjoint runs for nsteps steps with `slots` checkpoint
 * slots (the initial state included; a budget of B bytes gives
 * floor(B / snapshot bytes) slots, a snapshot being the state's 26
 * distributions in its storage format), recomputation and the terminal state
 * included: the same schedule, not run.  For planning a budget; no counterpart
 * in the reference.  -1 if nsteps or slots is below 1. */
long long lbm_adjoint_forward_steps(long long nsteps, int slots);

/* Largest box lbm_stats_noalloc accepts: 512^3 nodes. */
#define LBM_NOALLOC_MAX_NODES 134217728LL
/* Number of doubles lbm_stats_noalloc writes. */
#define LBM_STATS_RAW_VALUES 16

/* lbm_stats for callers that cannot allocate device memory.  No counterpart
 * in the reference (its statistics run on host copies of the fields).
 *
 * Meant for in-situ analysis and monitoring code that runs inside another
 * program's time loop: there the device memory belongs to the host
 * application's own pool allocator, and cudaMalloc / cudaFree are not allowed
 * (they take memory outside that budget and synchronise the whole device).
 * The caller passes what it already owns: the five fields on the device
 * (nx*ny*nz floats each, x fastest; only nx, ny, nz, device and the physical
 * parameters of p are used) and raw_out, a device buffer of
 * LBM_STATS_RAW_VALUES doubles.  The call allocates nothing; it queues two
 * kernels on `stream` (a cudaStream_t, NULL for the legacy default stream)
 * and returns.  raw_out then receives, in this order:
 *   0 max |u|^2 and 1 the number of nodes with phi >= 0, over the reference's
 *   region (planes x = 0, nx-1 and y = 0, ny-1 skipped); 2..4 sum of u over
 *   those phi >= 0 nodes; 5, 6 sum of the pressure over phi >= 0 / phi < 0
 *   nodes of that region; 7 sum phi; 8 sum rho; 9..11 sum rho u;
 *   12 number of nodes with phi >= 0; 13 max |u|^2; 14 number of nodes with a
 *   non-finite value (full domain for 7..14); 15 zero.
 * The per-block partial sums use a 1 MiB array in the library's static device
 * memory, which every GPU that loads the library keeps until the process
 * exits.  That array bounds the box: more than LBM_NOALLOC_MAX_NODES nodes is
 * rejected with LBM_EINVAL, and so are parameters whose constants cannot be
 * derived (tauRho, tauPhi or width not positive, rhoH == rhoL).  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress); under CUDA's lazy module loading (the default) that
 * first call is also when the driver loads the library's kernels and
 * reserves the array on that device, which is an allocation by the driver.
 * Make that first call during set-up, outside the time loop and before any
 * stream capture; later calls allocate nothing.  A cudaDeviceReset of the
 * device discards the array: do not call this entry point on that device
 * again.  All calls share the array: calls whose kernels can overlap on the
 * GPU (other streams, other host threads) race and must be ordered by the
 * caller.  Nothing in the array needs clearing between calls. */
int lbm_stats_noalloc(const lbm_params *p, const float *phi, const float *rho, const float *ux,
                      const float *uy, const float *uz, double *raw_out, void *stream);

/* ---- z-slab decomposition: one box over several contexts (GPUs) ----
 *
 * The reference splits the box in z over MPI ranks (src/vgrid.c:38-52) and
 * exchanges halo planes three times per step through host buffers
 * (src/main.cu:496-608 with src/pack_mpi*.cu, src/unpack_mpi*.cu,
 * src/mpiupdate*.c).  Here a z-slab context holds planes [z0, z0 + nz) of the
 * box, on its own device, with ghost planes around its fields; the fused step
 * needs two exchanges per step, both of whole planes:
 *   before every step (LBM_HALO_PRE): the two boundary planes of the seven f
 *     fields each way (the step's phi stencil reaches two planes out), and,
 *     before an odd step of the in-place (AA) g update, one boundary plane of
 *     the five g fields whose direction crosses the slab boundary;
 *   after an odd step (LBM_HALO_POST): the g values the step wrote into the
 *     ghost planes, back to the neighbour whose nodes they belong to.
 * A slab sends its "lo" buffer to the slab below and its "hi" buffer to the
 * slab above (periodic in z: the first slab's "below" is the last slab), and
 * unpacks what it receives from below as "lo" and from above as "hi".
 * LBM_HALO_PHI moves the boundary planes of the phi field for the statistics.
 * Slab contexts do not step with lbm_step and have no lbm_get_dist /
 * lbm_set_dist / snapshots / adjoint: they are made from and merged back into
 * a whole-box context. */
#define LBM_HALO_PRE 0
#define LBM_HALO_POST 1
#define LBM_HALO_PHI 2

/* Split the state of a whole-box context into nslabs z-slab contexts of
 * depths[k] >= 2 planes (summing to the box's nz; slab k starts at the sum of
 * the depths before it), slab k on device devices[k] (NULL: the whole
 * context's device), each with the whole context's parameters, storage map
 * and step count.  No counterpart in the reference (its ranks each build their
 * slab from the input files).  The whole context is left as it was. */
int lbm_split_z(lbm_ctx *whole, int nslabs, const int *depths, const int *devices, lbm_ctx **slabs);

/* One process per GPU, without the whole box on any device: each process
 * builds its own slab, planes [z0, z0 + depth) of the box p describes (p->nz
 * the whole box's planes, p->device this slab's device), from the bubble list,
 * as each rank of the reference builds its planes (src/init.c:39-59 with its
 * z offset; the planes next to the slab take phi from the geometry, as the
 * reference's ghost planes do).
 * The 16-bit storage map (one scale per distribution set) comes from maxima
 * over the whole box: lbm_slab_maxabs gives a slab's 26 maxima (|f_k|,
 * |g_i - w_i rho_mean|; zeros for FP32), the processes reduce them with MAX
 * (MPI_Allreduce, ncclAllReduce) and pass the result to
 * lbm_slab_init_bubbles (NULL is accepted for FP32 storage only).  The slabs
 * so made hold bit for bit what lbm_split_z of lbm_init_bubbles's whole box
 * holds.  Both synchronise. */
int lbm_slab_maxabs(const lbm_params *p, const float *bubbles, int nbubbles, int z0, int depth, float *maxabs);
int lbm_slab_init_bubbles(lbm_ctx **out, const lbm_params *p, const float *bubbles, int nbubbles, int z0,
                          int depth, const float *maxabs);

/* Gather the states of the slabs (as lbm_split_z made them, in order) back
 * into the whole-box context they came from (or one created with the same
 * parameters).  LBM_ESTATE if a slab still owes its neighbours the
 * LBM_HALO_POST exchange of an odd step.  Synchronises. */
int lbm_merge_z(lbm_ctx *const *slabs, int nslabs, lbm_ctx *whole);

/* nsteps steps of the whole box held by the slabs, with every exchange done
 * by device-to-device copies between the slabs' buffers (peer copies across
 * devices), ordered by events on the slabs' streams: the one-process driver
 * of the protocol above.  The phi, rho, u fields are written on the last step.
 * Asynchronous (lbm_sync each slab, or lbm_merge_z). */
int lbm_slab_step(lbm_ctx *const *slabs, int nslabs, int nsteps, float grav);

/* For one slab per process: the bytes of one side's buffer for a phase at the
 * slab's current step (0 when the phase has nothing to move: LBM_HALO_POST
 * after an even step), and the copies between the slab's planes and the
 * caller's device buffers (send_lo / send_hi, recv_lo / recv_hi, that many
 * bytes each), queued on the slab's stream.  A process moves the buffers to
 * its neighbours (NCCL send / recv, MPI, ...) between pack and unpack. */
long long lbm_halo_bytes(const lbm_ctx *slab, int phase);
int lbm_halo_pack(lbm_ctx *slab, int phase, void *send_lo, void *send_hi);
int lbm_halo_unpack(lbm_ctx *slab, int phase, const void *recv_lo, const void *recv_hi);

/* One step of a slab whose LBM_HALO_PRE exchange the caller has done; after
 * an odd step the LBM_HALO_POST exchange follows.  Writes the phi, rho, u
 * fields.  Asynchronous. */
int lbm_slab_step_local(lbm_ctx *slab, float grav);

/* The same step in two parts, so that the halo planes move while the slab
 * computes: lbm_slab_step_interior steps planes [2, nz - 2), which read
 * nothing the LBM_HALO_PRE exchange brings and write nothing it moves, and
 * may be queued between lbm_halo_pack and lbm_halo_unpack of that exchange
 * (and while the last step's LBM_HALO_POST exchange is still under way);
 * lbm_slab_step_boundary steps planes [0, 2) and [nz - 2, nz) after the
 * unpack (and after the LBM_HALO_POST exchange of the last step).  Once
 * each, in that order (LBM_ESTATE otherwise).  Asynchronous.  lbm_slab_step
 * runs its steps this way. */
int lbm_slab_step_interior(lbm_ctx *slab, float grav);
int lbm_slab_step_boundary(lbm_ctx *slab, float grav);

/* The 16 raw FP64 sums and maxima behind lbm_stats_out of a context's phi,
 * rho, u fields (layout of lbm_stats_noalloc's raw_out), for combining over
 * slabs: sums add and entries 0 and 13 (max |u|^2) take the maximum, the FP64
 * counterpart of the reference's MPI_Reduce of its statistics
 * (src/stats.c:57-58).  A slab's pressure sums need the phi planes around
 * it: do the LBM_HALO_PHI exchange first.  Synchronises. */
int lbm_stats_raw(lbm_ctx *c, double *raw);

/* lbm_stats_out of a whole box (p: its parameters, steps: its step count)
 * from raw statistics combined over its slabs (nraw sets of 16, combined
 * here; or one set the caller already reduced across processes). */
int lbm_stats_combine(const lbm_params *p, long long steps, const double *raw, int nraw, lbm_stats_out *s);

/* Statistics of the whole box held by the slabs: the LBM_HALO_PHI exchange,
 * lbm_stats_raw of each slab and lbm_stats_combine.  Synchronises. */
int lbm_slab_stats(lbm_ctx *const *slabs, int nslabs, lbm_stats_out *s);

/* Checkpoint / resume (no counterpart in the reference, whose VTK files are
 * output only): a snapshot of the context's state in its native form (the
 * current f_0 and f_1..f_6, g in its AA layout, the five moment fields, the
 * 16-bit storage map, the step count), into caller-owned host memory of
 * lbm_state_bytes bytes.  lbm_load_state restores it into a context of the
 * same box and storage format (created with the same parameters); stepping on
 * from there gives bit for bit what the saved context would have given.
 * LBM_EINVAL for a buffer that is not a snapshot or another box or format.
 * Both synchronise. */
long long lbm_state_bytes(const lbm_ctx *c);
int lbm_save_state(lbm_ctx *c, void *buf);
int lbm_load_state(lbm_ctx *c, const void *buf);

/* Steps taken since lbm_init. */
long long lbm_steps_done(const lbm_ctx *c);

/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work around lbm_step. */
void *lbm_stream(const lbm_ctx *c);

/* Wait for all work queued on the context.  LBM_ETIMEOUT if a step kernel gave
 * up one of its bounded waits for staged data (the step's results are then
 * not valid; the context's error flag stays set). */
int lbm_sync(lbm_ctx *c);

/* Failure-path self-test, no counterpart in the reference: one block waits,
 * with the step kernel's bounded wait, on a barrier that nothing completes; the
 * wait gives up, sets the context's error flag, and the error reaches the host
 * as it would from a step.  Returns LBM_ETIMEOUT (the expected outcome) after
 * clearing the flag, so the context stays usable; LBM_ESTATE if the wait did
 * not give up.  Synchronises. */
int lbm_wait_selftest(lbm_ctx *c);

/* Release the context and all its device memory.  NULL is a no-op. */
void lbm_destroy(lbm_ctx *c);

/* Text for a status code. */
const char *lbm_strerror(int code);

/* Detail of the last failure on this thread (CUDA error text, file name, ...). */
const char *lbm_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
