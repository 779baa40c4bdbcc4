/*
 * smob.h — C ABI of the GB300 sphere mobility library (libsmob.so).
 *
 * One context holds one or more independent mobility problems (a "batch"); each
 * problem is a set of rigid spheres whose surface densities live on the
 * (p+1) x (2p+2) Gauss-Legendre x uniform grid of each sphere. The context owns a
 * CUDA stream and all device memory; every call is synchronous with respect to the
 * host unless its name ends in _async. All entry points return an smob_status and
 * never throw; smob_last_error() gives the message of the last failure on the
 * calling host thread. A context is not re-entrant: use one context per host thread
 * (the reference operator keeps mutable scratch and is not re-entrant either,
 * BIE/SphereSTKSHOperator.hpp:123-157).
 *
 * Vector layouts follow the reference:
 *   - grid vectors: 3M doubles, interleaved (x,y,z) per point, spheres concatenated
 *     in input order, points of a sphere in the order j*(2p+2)+k (theta ring j from
 *     north to south, phi index k), poles excluded (Sphere/Shexp.cpp:206-271,
 *     BIE/SphereSTKSHOperator.cpp:83-122);
 *   - rigid-body vectors: 6N doubles (fx,fy,fz,tx,ty,tz) in, (vx,vy,vz,wx,wy,wz) out
 *     per sphere (BIE/SphereSTKMobMat.cpp:174-192,261-285);
 *   - spectral coefficients (smob_sh_* entry points): per sphere 3(p+1)(p+2) doubles,
 *     the project's own layout: three blocks [radial | surface-gradient | toroidal],
 *     each (p+1)(p+2)/2 complex numbers (re,im), n-major with m = 0..n, for the
 *     vector spherical harmonics Y r, grad_s Y, r x grad_s Y of the body frame with
 *     orthonormal Y_n^m without Condon-Shortley phase. The reference's SCTL layout
 *     has the same size; its exact convention is not reproduced.
 *   - quaternions: (w,x,y,z) per sphere, rotating the body frame into the lab frame.
 */
#ifndef SMOB_H
#define SMOB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct smob_ctx smob_ctx;

typedef enum {
    SMOB_OK = 0,
    SMOB_ERR_ARG = 1,          /* invalid argument (sizes, null pointers, overlapping spheres, order range) */
    SMOB_ERR_CUDA = 2,         /* CUDA runtime failure (message has the CUDA error string) */
    SMOB_ERR_NOMEM = 3,        /* device memory could not be allocated */
    SMOB_ERR_NOT_CONVERGED = 4,/* solve stopped at its iteration limit (outputs are still written) */
    SMOB_ERR_NONFINITE = 5,    /* NaN/Inf met in inputs or in the Krylov recurrence */
    SMOB_ERR_STATE = 6,        /* call not valid in the context's current state */
    SMOB_ERR_NO_DEVICE = 7     /* no usable CUDA device */
} smob_status;

typedef enum {
    SMOB_PREC_FP64 = 0,  /* every kernel in FP64 */
    SMOB_PREC_MIXED = 1, /* solves: FP32 operator inside high-precision iterative refinement (FP64 Arnoldi,
                            Givens; residuals with the float-float operator); operator calls: all FP32 */
    SMOB_PREC_FLOAT_FLOAT = 2 /* FP64 sphere kernels with the far and near fields in float-float (hi+lo float
                                 pairs on the FP32 pipe, ~48 bits): the high-precision operator of MIXED;
                                 for solves, plain restarted GMRES with this operator throughout */
} smob_precision;

typedef struct {
    int n_spheres;
    const double* centers;  /* 3N */
    const double* radii;    /* N, > 0 */
    const double* quats;    /* 4N (w,x,y,z), or NULL for identity orientations */
    const int* orders;      /* N, spherical-harmonic order p per sphere, 1 <= p <= 32 */
    const int* problem;     /* N, problem index per sphere (non-decreasing, 0..P-1), or NULL: one problem */
    double viscosity;       /* fluid viscosity (same for all problems), > 0 */
} smob_geometry;

/* initial guess of a mobility solve (smob_solve_opts.warm_start) */
typedef enum {
    SMOB_WARM_NONE = 0,
    SMOB_WARM_LAST = 1,    /* the previous solution (the reference's xLast) */
    SMOB_WARM_RECYCLE = 2  /* the combination of up to 16 earlier solutions on this geometry that fits the new
                              force best (exact for a force in their span); the solve adds its own
                              solution to them (smob_recycle_info) */
} smob_warm_start;

typedef struct {
    double tol;        /* relative residual |b - A mu| / |b| target (mobilitySolver.yaml "Convergence Tolerance") */
    int restart;       /* Krylov vectors per cycle ("Num Blocks") */
    int max_iters;     /* total GMRES iterations ("Maximum Iterations") */
    int precision;     /* smob_precision */
    int warm_start;    /* smob_warm_start: 0 zero initial guess; 1 the previous solution of each problem
                          (SphereSTKMobMat.cpp:222); 2 recycled solutions (smob_recycle_info) */
    double inner_tol;  /* MIXED only: relative tolerance of each FP32 inner solve (<= 0: library default 1e-5) */
    int precond;       /* 0: none (the reference's unpreconditioned GMRES); 1: right preconditioner that inverts
                          every sphere's own I/2 + K_PV + L exactly (block diagonal in the spherical-harmonic
                          basis). Same solution to the tolerance, fewer iterations, different Krylov path. */
} smob_solve_opts;

typedef struct {
    int status;        /* smob_status of this problem */
    int iterations;    /* GMRES iterations (MIXED: summed over refinement sweeps) */
    int refinements;   /* MIXED: refinement sweeps; FP64: restart cycles */
    int operator_passes_fp64; /* high-precision operator applications (FP64 / float-float: including b and
                                 the final velocity; MIXED: fused residual + single-layer passes, one each) */
    int operator_passes_fp32; /* FP32 operator applications */
    double relres;     /* final true relative residual |b - A mu|/|b| computed in the high-precision operator */
    double bnorm;      /* |b| */
} smob_problem_stats;

/* ---- lifetime ---- */
smob_status smob_create(smob_ctx** ctx, const smob_geometry* geom, int device);
smob_status smob_destroy(smob_ctx* ctx);
const char* smob_last_error(void);
smob_status smob_version(int* major, int* minor);

/* ---- sizes and grid (SphereSTKSHOperator::getGridCoords/Norms/Weights, hpp:218-223) ---- */
smob_status smob_get_sizes(const smob_ctx* ctx, int* n_spheres, int* n_points, int* n_problems, int* n_near_pairs);
smob_status smob_get_grid(const smob_ctx* ctx, double* coords3m, double* norms3m, double* weights_m);
smob_status smob_get_near_pairs(const smob_ctx* ctx, int* trg, int* src);

/* ---- SphereSTKSHOperator (BIE/SphereSTKSHOperator.hpp:112-231), host pointers ---- */
/* Y = alpha * A X + beta * Y with A = 0.5 I + K + L, on n_cols columns of length 3M
 * (column-major, leading dimension 3M). Replaces SphereSTKSHOperator::apply (cpp:153-236). */
smob_status smob_apply(smob_ctx* ctx, const double* X, double* Y, int n_cols, double alpha, double beta,
                       int precision);
/* out += c_id*in + c_sl*S[in] + c_trac*K[in] (add-into). Replaces applyP2POP (cpp:262-485). */
smob_status smob_apply_p2p(smob_ctx* ctx, const double* in, double* out, double c_id, double c_sl, double c_trac,
                           int precision);
/* out += c_lop * L[in] (add-into). Replaces applyLOP (cpp:487-521). */
smob_status smob_apply_lop(smob_ctx* ctx, const double* in, double* out, double c_lop);
/* in-place projection onto each sphere's band-limited space. Replaces projectNullSpace (cpp:239-260). */
smob_status smob_project_null_space(smob_ctx* ctx, double* inout);

/* ---- kernel-level pieces for parity tests (host pointers, add-into) ---- */
/* far field over all sources except the target's own sphere and its near-pair source spheres; FP64
 * sums every pair, SMOB_PREC_MIXED (FP32) and SMOB_PREC_FLOAT_FLOAT read coarse equivalent sources for
 * well-separated sphere pairs at the context's tolerances (smob_set_far_compression) */
smob_status smob_far_field(smob_ctx* ctx, const double* in, double* out, double c_sl, double c_trac, int precision);
/* spectral evaluation of the near-pair source spheres at their targets (no direct subtraction): FP64,
 * FP32 (SMOB_PREC_MIXED: tensor cores or SIMT, smob_set_near_tc), or float-float arithmetic on the FP64
 * coefficients (SMOB_PREC_FLOAT_FLOAT, the kernel of the high-precision passes) */
smob_status smob_near_field(smob_ctx* ctx, const double* in, double* out, double c_sl, double c_trac, int precision);
/* per-sphere G2S / S2G in the layout above (Shexp::calcSpectralCoeff / calcGridValue, Shexp.cpp:342-447) */
smob_status smob_sh_g2s(smob_ctx* ctx, const double* grid3m, double* coeff);
smob_status smob_sh_s2g(smob_ctx* ctx, const double* coeff, double* grid3m);
smob_status smob_coeff_offsets(const smob_ctx* ctx, int* offsets /* N+1, in doubles */);

/* Traction far field that allocates no device memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc where they need the far field: a host application
 * that has reserved (nearly) all GPU memory for its own pool leaves nothing to allocate, and a
 * loop that applies the operator thousands of times cannot pay for cudaMalloc/cudaFree (cudaFree
 * synchronizes the device). Everything is passed as device pointers: coords/norms/density (3n),
 * weights (n), sphere id per point (n); out (3n) += -3/(4 pi) * sum over points j on other spheres
 * of r (r . f_j)(r . n_i)/r^5 with f_j = c * weights[j] * density[j], r = x_i - x_j (near-pair
 * spheres are not excluded; a point of another sphere that coincides with the target, r = 0, adds
 * nothing). stream: a cudaStream_t, or NULL for the default stream.
 * Limit: 1 <= n_points <= 40960, otherwise SMOB_ERR_ARG. The scratch (per-chunk partial sums) is
 * a fixed 7.5 MiB __device__ array that every GPU loading the library keeps until exit; all calls
 * on a device share it and it keeps the last call's contents, so calls that overlap on the GPU
 * (different streams, or host threads) race. The array's device address belongs to the CUDA context
 * of the current device: a call made outside stream capture looks it up (cudaGetSymbolAddress) for
 * the current context, so a device reset or a non-primary context is followed; a call made while
 * its stream is being captured uses the address that an earlier call in the same context looked up,
 * so make the first call in each context before any stream capture (otherwise SMOB_ERR_STATE). */
smob_status smob_far_traction_noalloc(const double* d_coords, const double* d_norms, const double* d_weights,
                                      const double* d_density, const int* d_sphere, int n_points, double c,
                                      double* d_out, void* stream);

/* ---- SphereSTKMobMat (BIE/SphereSTKMobMat.hpp:26-79) ---- */
/* force6N -> vel6N for every problem of the context; density3M (may be NULL) receives rho+mu
 * (getDensitySolution, hpp:76); stats (may be NULL) has one entry per problem.
 * Replaces SphereSTKMobMat::solveMob (cpp:146-286) and apply (cpp:98-144). */
smob_status smob_solve_mob(smob_ctx* ctx, const double* force6n, double* vel6n, double* density3m,
                           const smob_solve_opts* opts, smob_problem_stats* stats);
/* the same with device pointers (inputs already resident; no host copies) */
smob_status smob_solve_mob_device(smob_ctx* ctx, const double* d_force6n, double* d_vel6n, double* d_density3m,
                                  const smob_solve_opts* opts, smob_problem_stats* stats);
/* Y = alpha * M X + beta * Y for the mobility matrix M (6N x 6N), n_cols columns (SphereSTKMobMat::apply,
 * BIE/SphereSTKMobMat.cpp:98-144); X and Y are [n_cols][6N]. On a one-problem context the columns
 * are solved together as by smob_solve_mob_multi. */
smob_status smob_mob_apply(smob_ctx* ctx, const double* X, double* Y, int n_cols, double alpha, double beta,
                           const smob_solve_opts* opts);
/* ---- time stepping: the geometry update between mobility solves of a time loop
 * (SphereSystem::moveEuler -> Sphere::stepEuler, SRC/SphereSystem.cpp:386-398, Sphere/Sphere.cpp:367-373).
 * centre += v dt; orientation rotated by omega dt (rotation by |omega| dt about omega, composed on the
 * left, normalised). The context is rebuilt in place for the new geometry: grid points, normals and the
 * far-field copies on the device, near pairs and their metadata on the host (O(N) data). The previous
 * solution stays as the warm start of the next solve (smob_solve_opts.warm_start, SphereSTKMobMat.cpp:222).
 * vel6n: [N][6] (v, omega) as the solve returns it. Spheres of one problem that would overlap give
 * SMOB_ERR_ARG and leave the context unchanged. Every kernel result after an update equals, bit for
 * bit, that of a context created from the updated geometry. */
smob_status smob_step_euler(smob_ctx* ctx, const double* vel6n, double dt);
/* the same with the velocities in device memory (e.g. the output of smob_solve_mob_device) */
smob_status smob_step_euler_device(smob_ctx* ctx, const double* d_vel6n, double dt);
/* new centres [3N] and orientations [4N] (NULL: unchanged) for the same spheres, rebuilt as above */
smob_status smob_set_geometry(smob_ctx* ctx, const double* centers, const double* quats);
/* current centres [3N] and orientations [4N] (either may be NULL) */
smob_status smob_get_geometry(const smob_ctx* ctx, double* centers, double* quats);

/* ---- output files in the reference's formats
 * A density (3M host values, e.g. getDensitySolution) on every sphere's grid with both poles added,
 * one VTK XML piece per sphere (Sphere::writeVTU / writePVTU, Sphere/Sphere.cpp:322-365; Shexp::writeVTU,
 * Sphere/Shexp.cpp:96-204): <prefix>Sphere_<name>_r0_<postfix>.vtu and <prefix>Sphere_<name>_<postfix>.pvtu.
 * Pole values are the density's expansion at theta = 1e-6 and pi - 1e-6 (weight 0 there). */
smob_status smob_write_vtu(smob_ctx* ctx, const char* prefix, const char* postfix, const char* name,
                           const double* density3m);
/* sphere centres and radii as XYZ (SphereSystem::writeXYZ, SRC/SphereSystem.cpp:158-179); gids: N ids
 * or NULL for 0..N-1 */
smob_status smob_write_xyz(smob_ctx* ctx, const char* path, const int* gids, double time);

/* Several right-hand sides on one geometry: the columns SphereSTKMobMat::apply solves one after
 * another with solveMob (BIE/SphereSTKMobMat.cpp:129-143), solved together, each with its own
 * Krylov space and stopping test. force6n [n_rhs][6N], vel6n [n_rhs][6N], density3m [n_rhs][3M] or
 * NULL, stats [n_rhs] or NULL. By default the columns are a batch of copies of the problem with the
 * context's own settings: every column's result equals bit for bit a smob_solve_mob of that column
 * alone. With smob_set_multi_shared_pairs(ctx, 1) the far field evaluates each grid-point pair once for
 * all columns instead (grid targets, every float-float pair); a column then equals its single solve
 * with smob_set_far_tile(ctx, 1), the coarse targets off and the float-float tolerance 0. The context
 * must hold one problem. Internal copies of the geometry are kept on the context per column count (at
 * most 4 counts). */
smob_status smob_set_multi_shared_pairs(smob_ctx* ctx, int on);
/* Far field from coarse equivalent sources. For a well-separated pair of spheres the far field of the
 * source sphere's grid sources is evaluated from equivalent sources on a coarser grid of the same
 * sphere: its grid sources projected onto the spherical harmonics of degree <= pe and re-weighted with
 * the order-pe quadrature, which reproduces the far field to ~(a_s / r_min)^(pe+1) relative (r_min:
 * distance from the source centre to the nearest target point). Each source sphere gets the coarse
 * orders its far targets need for the tolerance (relative to the sphere's own contribution; the
 * measured error stays within a small factor of it, below 3.4 eps over orders 8-24). eps sets
 * it for the FP32 operator passes (SMOB_PREC_MIXED inner solves and final velocity correction; default
 * 1e-5), eps_hp for the float-float passes (the MIXED refinement residuals and high-precision single
 * layer, SMOB_PREC_FLOAT_FLOAT; at most 1e-9). By default eps_hp follows the solves: 1e-9 at creation,
 * tightened once to a tenth of a solve's tolerance (not below 1e-12) when a solve asks for less than
 * 1e-8 (both sets are rebuilt then; never loosened); once set here it stays as set. Near pairs, the own sphere and every FP64 pass keep the
 * direct sum over the grid points: the plain FP64 solve is the reference's smooth quadrature. The
 * reference evaluates this far field with an FMM (STKFMM, BIE/SphereSTKSHOperator.cpp:291-292,368-369).
 * A tolerance <= 0 turns that set off (the direct sum). Setting the tolerances empties the recycled
 * solutions (smob_recycle_info) and drops the several-column copies of the context. */
smob_status smob_set_far_compression(smob_ctx* ctx, double eps, double eps_hp);
/* Coarse targets (on by default): the target side of a well-separated pair compressed the same way.
 * The far field of the source sphere (its coarse or grid sources) is evaluated at the nodes of a
 * coarse order pt of the target sphere and interpolated to its grid with the same reproducing kernel
 * (exact for fields of degree <= pt on the sphere), pt chosen like pe with the target radius and one
 * order more (the target normal of the traction), and only where pt's grid has at most 7/10 of the
 * sphere's points. Applies to the FP32 passes (tolerance eps) and to the MIXED solve's fused
 * float-float pass (eps_hp); the several-column solves keep grid targets. Same empties and drops as
 * smob_set_far_compression. */
smob_status smob_set_far_coarse_targets(smob_ctx* ctx, int on);
/* the tolerance, coarse points held and (sphere, level) entries of the FP32 set (hp = 0) or the
 * float-float set (hp = 1) */
smob_status smob_far_compression_info(const smob_ctx* ctx, int hp, double* eps, int* coarse_points, int* entries);
/* target-source pairs of one FP32 far-field pass with the current tile: the direct sum's (every far
 * pair), the evaluated ones (grid or coarse targets against grid or coarse sources, as the kernels
 * choose them), and the multiply-adds of the coarse strengths and the coarse targets' interpolation
 * per pass */
smob_status smob_far_pairs(const smob_ctx* ctx, long long* direct, long long* evaluated, long long* coarse_macs);
/* the same for the FP32 set (hp = 0, what smob_far_pairs reports) or for the float-float set (hp = 1: the
 * pairs one fused float-float pass of a MIXED solve evaluates, each for both kernels) */
smob_status smob_far_pairs_set(const smob_ctx* ctx, int hp, long long* direct, long long* evaluated,
                               long long* coarse_macs);

/* Recycled solutions for a sequence of solves on one geometry, e.g. the collision solver's repeated
 * mobility solves, whose forces are combinations of a few contact forces (the reference keeps its
 * Krylov solver between solves for this, BIE/SphereSTKMobMat.cpp:232). A solve with warm_start
 * SMOB_WARM_RECYCLE starts from mu0 = U Q^T F: the columns of Q are the forces of earlier such solves,
 * orthonormalised per problem, and U holds their density corrections transformed alike. The
 * correction is linear in the force, so a force in the span of earlier ones (a repeated force, a
 * combination of contact forces already seen) starts at the tolerance of those solves; otherwise mu0
 * is the least-squares fit. The solve then adds its own (F, mu). At most 16 pairs are kept (then the
 * space starts again from the newest); a geometry update, or a solve of another precision, empties it.
 * MIXED columns also hold the solve's final residual and high-precision single layer (linear in the
 * force as well), so a MIXED solve whose force lies in the span knows its residual without an
 * operator pass and needs only FP32 work. count: pairs held; capacity: 16.
 * smob_recycle_clear forgets the recycled pairs and the previous solution (warm_start 1). */
smob_status smob_recycle_info(const smob_ctx* ctx, int* count, int* capacity);
smob_status smob_recycle_clear(smob_ctx* ctx);

smob_status smob_solve_mob_multi(smob_ctx* ctx, int n_rhs, const double* force6n, double* vel6n,
                                 double* density3m, const smob_solve_opts* opts, smob_problem_stats* stats);

/* ---- serving: a request loop with continuous batching (no counterpart in the reference, which
 * solves one system per time step inside SphereSystem::resolveCollision, SRC/SphereSystem.cpp:403-479).
 * Requests (one independent problem each) are queued FIFO in two queues, small requests (fewer than
 * 1e9 far-field pairs) and big ones; up to max_slots of them are on the GPU at once, each admitted
 * when a slot is free and its device-memory footprint (smob_request_bytes) fits in what the running
 * requests leave of hbm_budget_bytes. The small queue is served first and big requests hold at most
 * max_slots minus a quarter of the slots (at least one). Every request runs on its own
 * stream with its own device-resident Krylov state, so concurrent requests overlap on the device;
 * a request's result is the same alone or in any mix (each is solved exactly as if alone). */
typedef struct smob_server smob_server;
typedef struct {
    int device;
    int max_slots;           /* requests on the GPU at once */
    double hbm_budget_bytes; /* admission budget (<= 0: 64 GB) */
    int restart;             /* GMRES restart */
    int max_iters;           /* GMRES iteration limit per request */
    int precision;           /* smob_precision of every request */
    double inner_tol;        /* MIXED inner tolerance (<= 0: library default) */
    int graphs;              /* CUDA graphs in the request contexts: 0 off, 1 on, 2 big requests only
                                (see smob_set_graphs) */
} smob_server_opts;
typedef struct {
    int state;               /* 0 queued, 1 on the GPU, 2 done */
    int status;              /* smob_status of the solve (when done) */
    double t_submit, t_admit, t_done; /* seconds since the server started */
    double bytes;            /* admission footprint */
    smob_problem_stats stats;
    double t_ctx;            /* seconds since the server started: the request's context was ready (solve start) */
    int route;               /* SMs it ran on: 0 the whole device, 1 the small partition, 2 the big partition */
} smob_request_info;
typedef struct {
    int queued, running;
    long long completed;
    double bytes_in_use, peak_bytes, budget_bytes, uptime_s;
    int peak_running;
} smob_server_info;
/* The server keeps freed device memory in the device's stream-ordered pool (its release threshold set
 * to the maximum) instead of returning it to the driver at every synchronisation, and turns off the
 * pool's reuse of blocks through inserted cross-stream waits (cudaMemPoolReuseAllowInternalDependencies),
 * so one request's allocation never waits for another request's queued kernels.
 * SMOB_ERR_ARG (before any device work) for max_slots, restart or max_iters below 1, or graphs
 * outside 0..2. */
smob_status smob_server_create(smob_server** server, const smob_server_opts* opts);
smob_status smob_server_submit(smob_server* server, const smob_geometry* geom, const double* force6n, double tol,
                               long long* request_id);
smob_status smob_server_poll(smob_server* server, long long request_id, double* vel6n, smob_request_info* info,
                             int* done);
smob_status smob_server_wait(smob_server* server, long long request_id, double timeout_s, double* vel6n,
                             smob_request_info* info);
smob_status smob_server_release(smob_server* server, long long request_id);
smob_status smob_server_stats(smob_server* server, smob_server_info* info);
/* SM partition of the serving device (no counterpart in the reference): small_sms SMs (rounded up to the
 * device's partition granularity, 8 on GB300) become a green context that small requests (fewer than
 * 1e9 far-field pairs) use while a big request is running; big requests run on a green context of the
 * remaining SMs; with no big request running a small one uses the whole device. Kernels already running
 * are never preempted, so without the partition a small request waits behind the long CTAs of big
 * ones. Results are the same bit for bit on any partition. 0 removes the partition. The server must be
 * idle (nothing queued or running), otherwise SMOB_ERR_STATE. */
smob_status smob_server_partition(smob_server* server, int small_sms);
/* SMs of the small and the big partition (0, 0 without a partition) */
smob_status smob_server_partition_info(smob_server* server, int* small_sms, int* big_sms);
smob_status smob_server_destroy(smob_server* server);
/* Builds the per-order host tables (grid, Legendre and twiddle tables, the near-field solid-harmonic
 * maps, the coarse equivalent-source maps of every coarse order below p) that the first context of an
 * order otherwise builds, for each listed order, and keeps them for the process. A server calls it for
 * the orders it expects so that no request pays for them (host work only; no device needed). */
smob_status smob_warm_orders(const int* orders, int n_orders);
/* admission footprint estimate (bytes of device memory) of one request; host-only arithmetic */
size_t smob_request_bytes(int n_spheres, const int* orders, int restart);

/* ---- device memory helpers for callers that time resident inputs ---- */
smob_status smob_device_alloc(smob_ctx* ctx, size_t bytes, void** ptr);
smob_status smob_device_free(smob_ctx* ctx, void* ptr);
smob_status smob_memcpy_h2d(smob_ctx* ctx, void* dst, const void* src, size_t bytes);
smob_status smob_memcpy_d2h(smob_ctx* ctx, void* dst, const void* src, size_t bytes);
smob_status smob_synchronize(smob_ctx* ctx);

/* ---- instrumentation ---- */
/* enable/disable CUDA-event timing of every kernel launch on the context's stream */
smob_status smob_profile_enable(smob_ctx* ctx, int on);
/* per-kernel totals since the last reset: name (NUL-terminated, truncated to name_len), launches, milliseconds */
smob_status smob_profile_count(const smob_ctx* ctx, int* n_kernels);
smob_status smob_profile_get(const smob_ctx* ctx, int i, char* name, int name_len, long long* launches, double* ms);
smob_status smob_profile_reset(smob_ctx* ctx);
/* total kernel launches issued by the library on this context since creation */
smob_status smob_launch_count(const smob_ctx* ctx, long long* launches);
/* CUDA graphs for the solves (default on). With the loop graph on (the default) a solve's whole
 * restart-cycle loop is one graph launch whose decisions run on the device: per-problem stop tests,
 * the Arnoldi steps (a switch over the step index inside a while node), the residual choice and the
 * next cycle (conditional graph nodes set by single-CTA decision kernels). With the loop graph off,
 * or where conditional nodes are unavailable, the host drives the cycles and replays captured blocks
 * of four steps, checking the per-problem stop flags between blocks. Results are the same bits. */
smob_status smob_set_graphs(smob_ctx* ctx, int on);
smob_status smob_set_loop_graph(smob_ctx* ctx, int on);
/* on: the loop graph is selected; available: building one has not failed on this context */
smob_status smob_loop_graph_info(const smob_ctx* ctx, int* on, int* available);
/* kernels run on this context since creation (graph nodes included) and launches issued from the host
 * (kernels launched outside graphs plus graph launches) */
smob_status smob_launch_stats(const smob_ctx* ctx, long long* kernels, long long* host_calls);
/* far-field tile shape chosen by the autotuner at smob_create: FP32 targets per thread (1, 2 or 4),
 * the measured milliseconds of the three variants (0 when the choice came from the process cache) */
smob_status smob_tuning(const smob_ctx* ctx, int* targets_per_thread, double* variant_ms, int* from_cache);
/* FP32 near field on the tensor cores (default 1): the contraction of each target point's solid
 * harmonics with a near source sphere's coefficient sets runs as a tcgen05 TF32 GEMM (3xTF32 split,
 * ~FP32 accuracy); 0 selects the SIMT kernel (same mathematics, FP32 multiply-adds). FP64 and
 * near-singular pairs always use the FP64 SIMT kernel. */
smob_status smob_set_near_tc(smob_ctx* ctx, int on);
/* The FP32 passes' coarse equivalent-source strengths (per (p, pe) map a GEMM [N_e x N_g] x [N_g x 3 per
 * sphere]) and their coarse-target interpolation (per map [N_g x N_e] x [N_e x 3 per entry]) as 3xTF32
 * GEMMs on the tcgen05 tensor cores (1, the default; k_coarse_src_tc: 128 coarse nodes x 16 spheres
 * per tile, its K chunks split over 4 CTAs and added in fixed order; k_ct_interp_tc: 128 grid points x
 * 16 entries) or as the SIMT FP32 GEMMs. mode: 1 both on the tensor cores (the default), 0 both on
 * the SIMT pipes, 2 only the strengths, 3 only the interpolation on the tensor cores. Both keep FP32-class accuracy (cfg2 far field 7.7e-7 and 4.8e-7 from FP64); each
 * problem's strengths are the same bits alone or in a batch with either. The tensor-core one needs
 * four partial strengths per coarse point of workspace. */
smob_status smob_set_coarse_tc(smob_ctx* ctx, int mode);
smob_status smob_coarse_tc_info(const smob_ctx* ctx, int* mode);
/* FP32 sphere operator (self terms of the FP32 passes) with the Legendre stage of its transforms on the
 * tensor cores: per order and m, the forward and inverse Legendre sums of up to 21 spheres as tcgen05
 * TF32 GEMMs (3xTF32 split), between per-sphere phi-DFT kernels (three launches per pass). Default 0:
 * the single SIMT kernel per sphere, which is faster at these sizes (the Legendre sums are a small part
 * of it). FP64 passes always use the FP64 SIMT kernel. */
smob_status smob_set_sphere_tc(smob_ctx* ctx, int on);
/* the current choices of smob_set_near_tc and smob_set_sphere_tc (either pointer may be NULL) */
smob_status smob_tc_info(const smob_ctx* ctx, int* near_tc, int* sphere_tc);
/* override the autotuner's choice (1, 2 or 4 FP32 targets per thread); every variant computes each
 * pair in the same order, so results change only by FP32 rounding in the sums of skipped sources */
smob_status smob_set_far_tile(smob_ctx* ctx, int targets_per_thread);
/* CUDA-event interval on the context's stream: mark records a start event; elapsed records an
 * end event, waits for it and returns the milliseconds since the last mark */
smob_status smob_timer_mark(smob_ctx* ctx);
smob_status smob_timer_elapsed(smob_ctx* ctx, double* ms);
/* writes `bytes` of a scratch buffer on the context's stream (used to evict L2 between timings) */
smob_status smob_flush_l2(smob_ctx* ctx, size_t bytes);
/* FP32 / FP64 FMA issue rate of a device in TFLOP/s (independent FMA chains): the SIMT roofline
 * denominators of the far-field kernels, measured in the same run */
smob_status smob_measure_fma_peaks(int device, double* fp32_tflops, double* fp64_tflops);

#ifdef __cplusplus
}
#endif
#endif /* SMOB_H */
