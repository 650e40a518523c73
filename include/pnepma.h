/*
 * pnepma.h -- C ABI of the GB300 PN-moment transport solve (forward k-ratio functional and
 * its adjoint gradient).
 *
 * The reference exposes this path as Julia methods with no foreign-function layer; the entry
 * points below are what a Julia shim binds with ccall to replace the methods at these places in
 * the reference (the callers, scripts/reconstructions_1d.jl:154, scripts/sensitivities_1d.jl:126-127
 * and scripts/2d_full_reconstruction_test.jl:138-147, reach them through Zygote):
 *
 *   pn_create            <- ForwardPNProblem{N,T}(...) / AdjointPNProblem(frwd)
 *                           pn_solver/pn_problem.jl:72-136 (matrices, boundary source, tables)
 *   pn_forward           <- calc_intensities(problem, m, x_rays, detector_position)
 *                           pn_solver/pn_intensities.jl:325-351
 *   pn_adjoint           <- the pullback of the Zygote.@adjoint of calc_intensities
 *                           pn_solver/pn_intensities.jl:353-413 (returns rho_bar, NOA_bar, ACS_bar;
 *                           the material pullbacks of :406-409 stay with the caller)
 *   pn_generation_field  <- calc_x_ray_generation_field, pn_solver/pn_intensities.jl:189-212
 *   pn_step              <- step_pn!(problem, rho, u, du, E, dE), pn_solver/pn_intensities.jl:16-30
 *                           (StaRMAP.step_pde!, starmap/src/solver.jl:171-196)
 *
 * Conventions
 *   - Units are the reference's calculation units: cm, g, eV (pn_solver/units.jl).
 *   - Class order is eee, eeo, eoe, eoo, oee, oeo, ooe, ooo (starmap/src/even_odd_classification.jl:19);
 *     class c has parity bits (ox, oy, oz) = (c>>2 & 1, c>>1 & 1, c & 1).
 *   - A class grid has M_d points along an axis where it is even, M_d + 1 (two ghost points)
 *     where it is odd, and 1 along a singleton axis (n_points[d] == 1).
 *   - Per-cell vectors are stored as the reference's Array{MVector} arrays are laid out in memory:
 *     the vector index fastest, then x, then y, then z.  Classes are concatenated in class order.
 *   - All functions return a pn_status; none aborts or throws across the ABI.  After an error,
 *     pn_last_error(handle) describes it.
 *   - A handle is used by one thread at a time; distinct handles may be used concurrently.
 *     The caller owns every host buffer; the library owns device memory.
 */
#ifndef PNEPMA_H
#define PNEPMA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PN_ABI_VERSION 1

typedef enum pn_status {
  PN_OK = 0,
  PN_ERR_INVALID = -1,       /* malformed descriptor or argument */
  PN_ERR_UNSUPPORTED = -2,   /* P_N order or layout not compiled into the library */
  PN_ERR_CFL = -3,           /* energy step above the stability estimate (only with PN_FLAG_CHECK_CFL) */
  PN_ERR_NO_MEMORY = -4,     /* device allocation failed or memory budget exceeded */
  PN_ERR_DIVERGED = -5,      /* a non-finite value appeared in the solution */
  PN_ERR_TIMEOUT = -6,       /* a bounded device-side wait ran out */
  PN_ERR_CUDA = -7,          /* CUDA runtime error */
  PN_ERR_STATE = -8,         /* call out of order (e.g. adjoint before forward) */
  PN_ERR_NO_DEVICE = -9      /* no CUDA device is available */
} pn_status;

typedef enum pn_precision {
  PN_FP64 = 0,   /* "plain" method: state, stencil and accumulators in FP64 */
  PN_FP32 = 1    /* state and stencil in FP32, intensity/gradient accumulators in FP64 */
} pn_precision;

enum pn_flags {
  PN_FLAG_CHECK_FINITE = 1,  /* report PN_ERR_DIVERGED when the intensities are not finite */
  PN_FLAG_CHECK_CFL = 2      /* reject descriptors whose energy step exceeds cfl_limit */
};

/*
 * Problem descriptor.  Everything the solve needs except the material fields.  The caller
 * evaluates the physical data (stopping power, transport coefficients, ionisation cross-sections,
 * beam) at the energies of the march and passes them as tables, exactly as the reference's
 * update_problem! would evaluate them (pn_solver/pn_problem.jl:157-249).
 *
 * Energy march: dE = (E_initial - E_cutoff) / n_steps; forward step i (1-based) goes from E_{i-1}
 * to E_i with coefficients at E_{i-1} - dE/2 (pn_intensities.jl:341-349).  Adjoint iteration
 * j = 0..n_steps-1 handles tape state n_steps - j at energy Ea_j (Ea_0 = E_cutoff, Ea_{j+1} =
 * Ea_j + dE); iteration j == n_steps is the final accumulation at the initial state
 * (pn_intensities.jl:391-404).
 */
typedef struct pn_desc {
  int32_t abi_version;       /* PN_ABI_VERSION */
  int32_t order;             /* P_N order N */
  int32_t n_points[3];       /* M per axis; 1 marks a singleton axis */
  int32_t n_elements;        /* n_e */
  int32_t n_xrays;           /* n_r */
  int32_t n_steps;
  int32_t precision;         /* pn_precision */
  int32_t checkpoint_stride; /* adjoint tape: K >= 1 keeps every K-th state and recomputes the rest
                                (1 keeps all); 0 keeps all while that fits in 2 GiB, else every
                                ceil(sqrt(n_steps))-th */
  int32_t flags;             /* pn_flags */
  int32_t reserved;
  double  h[3];              /* grid steps (1.0 on a singleton axis) */
  double  delta_e;           /* dE */
  double  dvol;              /* h_x h_y h_z */
  double  cfl_limit;         /* largest admissible dE when PN_FLAG_CHECK_CFL is set */
  const int32_t* xray_element;   /* [n_r] element index (0-based) emitting each line */

  /* advection blocks A_d[c], dense n_c x n_switch(c,d), row-major, for d = x,y,z and c = 0..7 in
     that nesting; blocks of classes with no moments are empty.  The sparsity must match the
     closed form of pn_solver/pn_matrices.jl:146-152 for this order (checked at pn_create). */
  const double* advection;
  /* boundary blocks for classes odd in d, same nesting, dense n_c x n_switch(c,d):
     forward L*A (pn_matrices.jl:277-284) and adjoint -L'*A (pn_matrices.jl:286-293) */
  const double* boundary_fwd;
  const double* boundary_adj;
  /* beam source on the right x face (gx_temp[eo][2,:,:], pn_problem.jl:192-203) for the classes
     odd in x (oee, oeo, ooe, ooo in that order): [class][z][y][moment] */
  const double* beam_face;

  /* forward march, step i = 0..n_steps-1 (coefficients at E_i - dE/2 with E_0 = E_initial) */
  const double* fwd_s;       /* [step][e]      s_e                          (update_coefficients!) */
  const double* fwd_c;       /* [step][e][l]   c_{e,l} = -s_e' - (tc_l - tc_0), l = 0..N      */
  const double* fwd_bc;      /* [step]         (Phi(E+dE) - Phi(E)) / dE   (update_boundary_condition!) */
  const double* fwd_sigma;   /* [n_steps+1][r] sigma_r(E_i), i = 0..n_steps */
  const double* fwd_weight;  /* [n_steps+1]    int_fac of each accumulation */

  /* adjoint march, iteration j = 0..n_steps */
  const double* adj_int_s;   /* [j][e]    forward s_e(Ea_j) */
  const double* adj_int_c;   /* [j][e][l] forward c_{e,l}(Ea_j) */
  const double* adj_int_bc;  /* [j]       forward beam weight at Ea_j */
  const double* adj_sigma;   /* [j][r]    sigma_r(Ea_j) */
  const double* adj_weight;  /* [j]       int_fac */
  const double* adj_src_sigma; /* [j][r]  sigma_r(Ea_j + dE/2), j < n_steps */
  const double* adj_s;       /* [j][e]    s_e(Ea_j + dE/2), j < n_steps */
  const double* adj_c;       /* [j][e][l] adjoint c_{e,l} = -(tc_l - tc_0) at Ea_j + dE/2 */
} pn_desc;

/* Sizes the caller must allocate, derived from a descriptor. */
typedef struct pn_sizes {
  int32_t n_moments[8];      /* moments per class */
  int32_t shape[8][3];       /* class grid (nx, ny, nz) including ghost points */
  int64_t n_rho;             /* doubles in a rho / rho_bar buffer (all 8 classes, n_e per point) */
  int64_t n_eee_cells;       /* cells of the eee grid */
  int64_t n_noa;             /* n_eee_cells * n_e */
  int64_t n_acs;             /* n_eee_cells * n_r */
  int64_t n_state;           /* doubles of a full state (all 8 classes, moments per point) */
  int64_t n_beam_face;       /* doubles expected in beam_face */
  int64_t n_advection;       /* doubles expected in advection */
  int64_t n_boundary;        /* doubles expected in boundary_fwd (and boundary_adj) */
  int64_t device_bytes;      /* device memory pn_create will allocate */
} pn_sizes;

typedef struct pn_handle pn_handle;

/* Fill *sizes for a descriptor (no device work).  Replaces nothing in the reference; it lets a
   shim allocate the buffers the reference would have allocated itself. */
int pn_query_sizes(const pn_desc* desc, pn_sizes* sizes);

/* Validate the descriptor, copy its tables to the device and allocate the state and tape.
   Replaces the construction of ForwardPNProblem / AdjointPNProblem (pn_problem.jl:72-136). */
int pn_create(const pn_desc* desc, pn_handle** out);

/* Forward march and intensities.  rho: [n_rho] component densities on all 8 class grids
   (component_densities(m, gspec), pn_material_utils.jl:74-83); noa: [n_eee_cells][n_e] number of
   atoms (x_ray_intensities.jl:43-55); acs: [n_eee_cells][n_r] absorption factors
   (x_ray_intensities.jl:115-128); intensities: [n_r] out.  Keeps the forward tape on the device
   for a following pn_adjoint.  Replaces calc_intensities (pn_intensities.jl:325-351). */
int pn_forward(pn_handle* h, const double* rho, const double* noa, const double* acs,
               double* intensities);

/* Adjoint march for cotangent intensities_bar [n_r] after pn_forward on the same handle.
   Outputs (overwritten): rho_bar [n_rho] (zero on ghost points and inactive classes),
   noa_bar [n_eee_cells][n_e], acs_bar [n_eee_cells][n_r].  Replaces the body of
   calc_intensities_pullback up to the material pullbacks (pn_intensities.jl:381-405). */
int pn_adjoint(pn_handle* h, const double* intensities_bar, double* rho_bar, double* noa_bar,
               double* acs_bar);

/* Same as pn_forward / pn_adjoint with device pointers (device-resident inputs and outputs),
   ordered on the CUDA stream `stream` (a cudaStream_t, NULL for the legacy default stream). */
int pn_forward_device(pn_handle* h, const double* rho, const double* noa, const double* acs,
                      double* intensities, void* stream);
int pn_adjoint_device(pn_handle* h, const double* intensities_bar, double* rho_bar,
                      double* noa_bar, double* acs_bar, void* stream);

/* x-ray generation field: out [n_eee_cells][n_r] = sum over steps of u_eee[cell,0] dE sigma_r w
   (pn_intensities.jl:189-212 with integrate_step_and_add_x_ray_generation!,
   x_ray_intensities.jl:226-234). */
int pn_generation_field(pn_handle* h, const double* rho, double* field);

/* One forward energy step of the state held by the handle, in place (step_pn!,
   pn_intensities.jl:16-22): uses the coefficients of forward step `step` (0-based).
   pn_set_state / pn_get_state move the state in the reference's layout: [n_state] doubles,
   classes concatenated, moments fastest.  Ghost points are updated as the reference updates
   them, except points that are ghosts along two or more axes and the classes odd in a singleton
   axis: no stencil reads those, and they are returned as zero. */
int pn_set_state(pn_handle* h, const double* rho, const double* state);
int pn_step(pn_handle* h, int32_t step);
int pn_get_state(pn_handle* h, double* state);

/* Forward intensity march that allocates nothing (no counterpart in the reference).
   For callers that cannot allocate device memory while they solve -- their GPU memory is owned by
   another allocator that has reserved it, or they run a latency-bound loop where cudaMalloc /
   cudaFree would synchronise the device.  Same result as pn_forward (FP64 descriptors only), but
   rho, noa, acs and intensities are device pointers owned by the caller, the work is ordered on
   `stream` (a cudaStream_t, NULL = legacy default stream) without synchronising, and every
   scratch buffer comes from one library-owned device array of PN_NOALLOC_SCRATCH_BYTES per GPU,
   held by every GPU that loads the library until the process exits.  Problems whose scratch does
   not fit are rejected with PN_ERR_NO_MEMORY (message from pn_last_error(NULL)).  The first call
   on a device looks up the array's device address (cudaGetSymbolAddress) and should come before
   any stream capture.  All calls share the array: calls whose work overlaps on the GPU race and
   must be serialised by the caller.  The descriptor is checked as pn_create checks it (same
   errors, PN_FLAG_CHECK_CFL and PN_FLAG_CHECK_FINITE honoured; the latter synchronises `stream`).
   The descriptor's host tables are read by asynchronous host-to-device copies on `stream`:
   pageable tables may be reused once the call returns, page-locked (pinned or registered) tables
   must stay unchanged until `stream` has reached this call's work. */
#define PN_NOALLOC_SCRATCH_BYTES (64u << 20)
int pn_forward_noalloc(const pn_desc* desc, const double* rho, const double* noa, const double* acs,
                       double* intensities, void* stream);

/* Facts about a created handle (diagnostics; no counterpart in the reference). */
typedef struct pn_handle_info {
  int32_t checkpoint_stride;   /* stride in use (1 = every state kept) */
  int32_t precision;
  int64_t device_bytes;        /* device memory held by the handle */
  int64_t forward_kernels;     /* kernel launches of one pn_forward(_device) call */
  int64_t adjoint_kernels;     /* kernel launches of one pn_adjoint(_device) call */
} pn_handle_info;

int pn_query_handle(const pn_handle* h, pn_handle_info* info);

void pn_destroy(pn_handle* h);

/*
 * Batched solves (no counterpart in the reference, whose scripts call calc_intensities once per
 * beam position and energy, scripts/2d_full_reconstruction_test.jl:104-149).  Many descriptors,
 * possibly of different orders, grids, element counts and step counts, marched together: one
 * kernel launch per sub-step covers every solve of one order.  All descriptors must share one
 * precision; the coupling blocks must be the closed form of pn_matrices.jl:146-152.  Inputs and
 * outputs are arrays (one entry per solve, in descriptor order) of device pointers with the same
 * layouts as pn_forward / pn_adjoint; work is ordered on `stream` without synchronising.
 */
typedef struct pn_batch pn_batch;

typedef struct pn_batch_options {
  int64_t memory_budget;      /* bytes of device memory for the tapes; 0 = half of the free memory */
  int32_t checkpoint_stride;  /* 0 = the tape that recomputes the fewest steps within the budget
                                 (every state when it fits; else the first A states in full and
                                 every K-th beyond them); K >= 1 forces stride K, no full head */
  int32_t flags;              /* pn_batch_flags */
} pn_batch_options;

enum pn_batch_flags {
  /* FP32 2D (x, y) and 3D groups run their sub-steps on TMA tiles (with sub-steps 3 and 1 of
     consecutive energy steps fused into one launch) unless this is set; the generic kernels give
     bit-identical states and gradients (for comparison and diagnosis) */
  PN_BATCH_GENERIC_KERNELS = 1,
  /* issue the kernels of every sweep on the caller's stream instead of capturing the sweeps as
     CUDA graphs at creation: cheaper for a batch that runs once (each call then launches 2-3
     kernels per energy step from the host) */
  PN_BATCH_DIRECT_LAUNCH = 2,
  /* test hook for the failure path of the bounded device-side waits (FP32 TMA groups): the first
     tile wait of the batch's first sub-step launch is reported as run out after it has completed,
     so the launch takes its timeout path (status PN_ERR_TIMEOUT, copies in flight drained, the CTA
     returns) without any copy in flight; that call's results are then incomplete.  Later calls
     run normally; the status word is cleared by every pn_batch_forward */
  PN_BATCH_TEST_EXPIRE_WAIT = 4,
  /* FP32 TMA groups: one persistent cooperative launch per sweep (batch_sweep_kernel), in which
     the tiles of a solve's steps wait on per-solve completion counters, instead of one kernel
     launch per sub-step (or fused pair) and per density integral.  Identical results; measured
     slower on the 2D P11 workload (each tile waits for its stores to land before it releases
     its counter), so off by default and one of the autotuner's choices */
  PN_BATCH_SWEEP_LAUNCH = 16,
  /* FP32 2D groups: parity tiles (both target classes of a parity at one 32 x 4 position, one
     36 x 5 box per neighbour class: a third less shared memory per target point) instead of one
     TMA tile per target class (a 32 x 4 box, a 40 x 4 x-neighbour box and a 32 x 5 y-neighbour
     box).  Identical results; measured as fast as the class tiles on the 2D P11 workload, so off
     by default and one of the autotuner's choices */
  PN_BATCH_PARITY_TILES = 32,
  /* bits 8..11: resident CTAs per SM of the persistent TMA tile kernels, 1..15 (0: as many as the
     shared memory and registers allow); fewer CTAs each walk more tiles.  One of the autotuner's
     choices (tiles per CTA) */
  PN_BATCH_CTAS_PER_SM_SHIFT = 8
};

typedef struct pn_batch_info {
  int32_t n_solves;
  int32_t n_groups;           /* one per distinct (order, set of active axes) */
  int32_t checkpoint_stride;  /* largest stride in use */
  int32_t tma_groups;         /* groups whose sub-steps stage their tiles with TMA */
  int64_t device_bytes;
  int64_t forward_kernels;    /* kernel launches of one pn_batch_forward */
  int64_t adjoint_kernels;    /* kernel launches of one pn_batch_adjoint */
  int64_t recomputed_steps;   /* forward energy steps one pn_batch_adjoint recomputes, all solves */
} pn_batch_info;

int pn_batch_create(const pn_desc* const* descs, int32_t n, const pn_batch_options* options, pn_batch** out);
int pn_batch_forward(pn_batch* b, const double* const* rho, const double* const* noa,
                     const double* const* acs, double* const* intensities, void* stream);
int pn_batch_adjoint(pn_batch* b, const double* const* intensities_bar, double* const* rho_bar,
                     double* const* noa_bar, double* const* acs_bar, void* stream);
/* Fills *info.  Returns PN_ERR_TIMEOUT when a bounded device-side wait of the latest
   pn_batch_forward or of the pn_batch_adjoint calls after it ran out (call it after that work has
   completed). */
int pn_batch_query(const pn_batch* b, pn_batch_info* info);
void pn_batch_destroy(pn_batch* b);

/*
 * Served solves (no counterpart in the reference: its reconstruction loops call calc_intensities
 * and the pullback one beam position and energy at a time, scripts/reconstructions_1d.jl:56-185,
 * scripts/2d_full_reconstruction_test.jl:104-234).  A request is a list of solves -- e.g. one
 * Gauss-Newton iteration's beam positions x energies, forward and adjoint -- submitted from any
 * thread.  One scheduler thread per server admits waiting requests in arrival order as wave slots
 * and room in the memory budget free up.  The request at the head of the queue and every later
 * waiting request of the same kind (precision, mode, and set of (order, active axes) of its
 * solves) become one batched wave (pn_batch_create's engine), and each wave runs on its own
 * streams, so requests admitted while others are on the GPU overlap with them.  Each solve's result does not
 * depend on which other solves share its wave.  All device memory of a wave (tables, tapes,
 * checkpoints, inputs, outputs) is carved from one allocation of memory_budget bytes made by
 * pn_server_create; releasing it never synchronises the device.
 *
 * Buffers are the caller's HOST buffers with the layouts of pn_forward / pn_adjoint.  The server
 * reads the descriptors, their tables and the inputs when it admits the request and writes the
 * outputs when the request completes: every pointer in the request must stay valid until
 * pn_poll or pn_wait reports the ticket done.  Inputs passed by the same pointer to several solves
 * of a wave are uploaded once.
 */
typedef struct pn_server pn_server;

typedef struct pn_server_options {
  int64_t memory_budget;      /* device bytes reserved for the waves; 0 = half of the free memory */
  int32_t max_waves;          /* waves on the GPU at once; 0 = 8 */
  int32_t max_wave_solves;    /* solves merged into one wave; 0 = 1024 */
  int32_t checkpoint_stride;  /* 0 = chosen per wave from its share of the budget */
  int32_t reserved[3];
} pn_server_options;

typedef struct pn_request {
  int32_t n_solves;
  int32_t adjoint;                        /* 1: forward then adjoint; 0: forward only */
  const pn_desc* const* descs;            /* [n_solves], one precision */
  const double* const* rho;               /* [n_solves] x [n_rho] */
  const double* const* noa;               /* [n_solves] x [n_eee_cells][n_e] */
  const double* const* acs;               /* [n_solves] x [n_eee_cells][n_r] */
  const double* const* intensities_bar;   /* [n_solves] x [n_r]; read when adjoint = 1 */
  double* const* intensities;             /* [n_solves] x [n_r] out */
  double* const* rho_bar;                 /* outs written when adjoint = 1 */
  double* const* noa_bar;
  double* const* acs_bar;
} pn_request;

typedef struct pn_ticket_info {
  int32_t done;       /* 1 once the outputs are written */
  int32_t status;     /* pn_status of the request once done */
  int32_t wave;       /* wave the request ran in; -1 while waiting */
  int32_t reserved;
  double queued_ms;   /* submission to admission (-1 while waiting) */
  double total_ms;    /* submission to outputs written (-1 until done) */
} pn_ticket_info;

typedef struct pn_server_info {
  int64_t memory_budget;
  int64_t bytes_in_use;
  int64_t peak_bytes;
  int64_t requests_submitted;
  int64_t requests_done;
  int64_t solves_done;
  int64_t waves_launched;
  int32_t waves_in_flight;
  int32_t max_waves_in_flight;   /* most waves on the GPU at once so far */
  int64_t wave_build_us;         /* host time spent building waves (tables, uploads, graphs), total */
} pn_server_info;

int pn_server_create(const pn_server_options* options, pn_server** out);
/* Queue a request; *ticket identifies it.  Fails (PN_ERR_INVALID) only for a malformed request;
   device and budget errors are reported by pn_poll / pn_wait. */
int pn_submit(pn_server* s, const pn_request* req, uint64_t* ticket);
/* Non-blocking state of a ticket; a failed request's message goes to pn_last_error(NULL). */
int pn_poll(pn_server* s, uint64_t ticket, pn_ticket_info* info);
/* Block until the ticket is done (timeout_ms < 0: no limit) and return its status, or
   PN_ERR_TIMEOUT.  A failed request's message goes to pn_last_error(NULL). */
int pn_wait(pn_server* s, uint64_t ticket, int64_t timeout_ms);
int pn_server_query(pn_server* s, pn_server_info* info);
/* Requests not yet admitted fail with PN_ERR_STATE; running waves are completed first. */
void pn_server_destroy(pn_server* s);

/*
 * Material on the device: the solve's inputs from the material parameters, and the material
 * pullbacks of the gradient, so that neither the fields nor m_bar cross to the host.
 *
 *   pn_material_fields    <- component_densities(m, gspec)       pn_material_utils.jl:74-83
 *                            compute_number_of_atoms             x_ray_intensities.jl:43-55
 *                            compute_absorption_coefficients     x_ray_intensities.jl:100-128
 *   pn_material_pullback  <- component_densities_pullback        pn_material_utils.jl:85-91
 *                            compute_absorption_coefficient_pullback  x_ray_intensities.jl:131-153
 *                            compute_number_of_atoms_pullback    x_ray_intensities.jl:84-96
 *                            (the three calls at the end of calc_intensities_pullback,
 *                            pn_intensities.jl:406-409)
 *
 * Material models (pn_parametrizations/pn_material.jl): with p the parametrisation's value at a
 * point (n_e values, or n_e - 1 for an SC variant, whose last component is 1 - sum of the others):
 *   MassConcentration  rho = p                              (:56-77; no SC variant)
 *   VolumeFraction     rho = p .* rho_pure                  (:79-134)
 *   LinearDensity      rho = p * dot(p, rho_pure)           (:137-197)
 *   MassFraction       rho = p / sum(p ./ rho_pure)         (:199-264)
 * Parametrisations: Const (pn_parametrization_const.jl), Boxed (pn_parametrization_boxed.jl:
 * piecewise constant on the boxes between slices, `embedding` outside) and Bilinear
 * (pn_parametrization_bilinear.jl with biliner_interp.jl:63-111: trilinear between knots, the
 * embedding value at knots outside the grid).
 * Parameter vector (the reference's param_vec order): Const: [n_par]; Boxed and Bilinear:
 * [z][y][x][n_par] over boxes or knots, then the embedding [n_par] (always present; its entries of
 * params_bar are the embedding's gradient, which a non-optimisable embedding ignores).
 */
typedef enum pn_material_model {
  PN_MAT_MASS_CONCENTRATION = 0,
  PN_MAT_VOLUME_FRACTION = 1,
  PN_MAT_LINEAR_DENSITY = 2,
  PN_MAT_MASS_FRACTION = 3
} pn_material_model;

typedef enum pn_parametrization_kind {
  PN_PAR_CONST = 0,
  PN_PAR_BOXED = 1,
  PN_PAR_BILINEAR = 2
} pn_parametrization_kind;

/* Slices (box boundaries) or knots along one axis.  Range form (`values` NULL): a StepRangeLen
   with Float64(ref), Float64(step), its offset (1-based index of ref) and length n; located by
   floor((x - ref) / step) (biliner_interp.jl:5-15).  Vector form (Boxed only): n increasing values
   located by the reference's linear search (biliner_interp.jl:18-36), under which a point on an
   interior slice belongs to the box below it. */
typedef struct pn_slices {
  int32_t n;
  int32_t offset;
  double ref;
  double step;
  const double* values;
} pn_slices;

typedef struct pn_material_desc {
  int32_t model;             /* pn_material_model */
  int32_t sc;                /* 1: the SC variant (not for MassConcentration) */
  int32_t parametrization;   /* pn_parametrization_kind */
  int32_t n_elements;        /* n_e */
  int32_t n_points[3];       /* the solve's pn_desc.n_points */
  int32_t n_xrays;           /* lines of the absorption factors (0: none) */
  int32_t n_int_points;      /* samples per absorption ray (the reference uses 100) */
  int32_t reserved;
  /* grid coordinates per axis x, y, z: the even points (n_points[d]) then the odd points
     (n_points[d] + 1; 1 on a singleton axis), as points(eo, gspec) yields them */
  const double* coords;
  pn_slices slices[3];       /* unused for Const */
  const double* rho_pure;    /* [n_e] VolumeFraction / MassFraction rho_pure, LinearDensity rho */
  const double* atom_mass;   /* [n_e] mass of one atom (g), the divisor of the number of atoms */
  const double* mac;         /* [n_r][n_e] mass absorption coefficients */
  double detector[3];        /* detector position x_d */
  double beam_x;             /* x coordinate of the beam position x_b */
} pn_material_desc;

typedef struct pn_material pn_material;

/* Validate the descriptor and copy its tables to the device; *n_params receives the length of
   the parameter vector (NULL allowed). */
int pn_material_create(const pn_material_desc* desc, pn_material** out, int64_t* n_params);

/* Device pointers, ordered on `stream` (a cudaStream_t, NULL = legacy default stream).  params:
   [n_params].  Outputs in pn_forward's layouts, each optional (NULL skips it): rho [n_rho] on all
   eight class grids, noa [n_eee_cells][n_e], acs [n_eee_cells][n_r]. */
int pn_material_fields(pn_material* m, const double* params, double* rho, double* noa, double* acs,
                       void* stream);

/* params_bar [n_params] (overwritten) = the parameter gradient of sum(rho_bar . rho) +
   sum(noa_bar . noa) + sum(acs_bar . acs), from pn_adjoint's outputs; acs is the forward's
   absorption factors.  Any of rho_bar, noa_bar and acs_bar may be NULL (acs then too).
   Accumulated with FP64 atomics: the summation order, hence the last bits, may vary between
   runs. */
int pn_material_pullback(pn_material* m, const double* params, const double* rho_bar,
                         const double* noa_bar, const double* acs, const double* acs_bar,
                         double* params_bar, void* stream);

void pn_material_destroy(pn_material* m);

/* Human-readable description of the last error on this handle (or, when h is NULL, of the last
   failed call in this thread that has no handle: pn_create, pn_query_sizes, pn_batch_*,
   pn_forward_noalloc, pn_server_*, pn_submit, pn_poll, pn_wait, pn_material_*).  Never NULL. */
const char* pn_last_error(const pn_handle* h);

/* Self-test of the FP32 exponential factor phi1(c) = (e^c - 1) / c used by the FP32 kernels
   (no counterpart in the reference): evaluates it and the expm1f(c) / c form for n arguments. */
int pn_selftest_phi1(int32_t n, const float* x, float* phi1_fast, float* phi1_ref);

/* Self-test of the FP64 exponential factor phi1(c) = (e^c - 1) / c of the FP64 kernels (no
   counterpart in the reference): evaluates it on the device for n arguments. */
int pn_selftest_phi1_f64(int32_t n, const double* x, double* phi1);

/* FP64 throughput probe (diagnostic; no counterpart in the reference): launches `blocks` blocks of
   256 threads, each thread running 8 independent FP64 FMA chains for `iters` iterations
   (blocks * 256 * iters * 16 flops) on `stream`; `out` is a device buffer of `blocks` doubles.
   The benchmark times it with events to measure the FP64 roofline of the plain path. */
int pn_probe_fp64_fma(int32_t blocks, int32_t iters, double* out, void* stream);

/* ABI version and the compiled P_N orders (bit N set when order N is available). */
int32_t pn_abi_version(void);
int64_t pn_compiled_orders(void);

#ifdef __cplusplus
}
#endif

#endif /* PNEPMA_H */
