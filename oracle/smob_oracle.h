/*
 * smob_oracle.h — FP64 CPU restatement of the reference's sphere mobility path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA product
 * (spheresimulator_gb300/csrc) and the timed CPU baseline. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs may load it. Nothing in the
 * product path links or calls it.
 *
 * Reference files restated here (paths inside wenyan4work/SphereSimulator):
 *   Sphere/Shexp.cpp:206-271      grid, quadrature weights, normals, quaternion rotation
 *   Sphere/Shexp.cpp:342-447      S2G / G2S vector spherical-harmonic transforms (SCTL Grid2VecSHC/VecSHC2Grid)
 *   Sphere/Shexp.cpp:503-624      spectral SL / traction evaluation (SCTL StokesEvalSL/KL/KSelf)
 *   BIE/SphereSTKSHOperator.cpp:262-485  applyP2POP (far field, self PV, identity, near corrections)
 *   BIE/SphereSTKSHOperator.cpp:487-521  applyLOP
 *   BIE/SphereSTKSHOperator.cpp:153-236  apply (Y = alpha*A*X + beta*Y)
 *   BIE/SphereSTKMobMat.cpp:146-286      solveMob
 *   MPI/NearInteraction.txx:430-447      near-pair rule
 *   mobilitySolver.yaml:3-16             GMRES settings (restarted GMRES, IMGS)
 *
 * Parity status: the spectral layer-potential evaluations are pinned to direct grid
 * quadrature at far targets exactly as Sphere/Shexp_test.cpp:109-524 does; the
 * SCTL coefficient layout is not reproduced (the project's own layout is documented
 * in include/smob.h), so comparisons with the reference are made in grid space.
 */
#ifndef SMOB_ORACLE_H
#define SMOB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sphere-level (Shexp) operations; quat is (w,x,y,z) or NULL for identity ---- */
int orc_grid_number(int p);                 /* (p+1)(2p+2) */
int orc_spectral_dof(int p);                /* 3(p+1)(p+2) doubles */
/* grid with poles removed: coords (3Ng, centre + a*R*yhat), norms (3Ng), weights (Ng) */
void orc_sh_grid(int p, double radius, const double* quat, const double* center, double* coords, double* norms,
                 double* weights);
void orc_gauss_legendre(int n, double* nodes, double* weights);
void orc_sh_g2s(int p, const double* quat, const double* grid3, double* coeff);
void orc_sh_s2g(int p, const double* quat, const double* coeff, double* grid3);
/* kind: 0 = single layer (on surface), 1 = exterior traction limit, 2 = interior traction limit,
 * 3 = principal value 0.5*(ext+int). Output on the sphere's own grid, lab frame. */
void orc_sh_self(int p, double radius, const double* quat, const double* coeff, int kind, double* grid3);
/* off-surface exterior evaluation at targets given relative to the sphere centre (lab frame).
 * sl_out (3nt) may be NULL; trac_out (3nt) needs trg_norm. */
void orc_sh_eval_exterior(int p, double radius, const double* quat, const double* coeff, int nt, const double* trg_rel,
                          const double* trg_norm, double* sl_out, double* trac_out);

/* ---- operator context ---- */
void* orc_create(int n_spheres, const double* centers, const double* radii, const double* quats, const int* orders,
                 double viscosity);
void orc_destroy(void* ctx);
int orc_num_points(void* ctx);
int orc_num_pairs(void* ctx);
void orc_get_pairs(void* ctx, int* trg, int* src);
void orc_get_grid(void* ctx, double* coords, double* norms, double* weights);
void orc_apply_p2p(void* ctx, const double* in, double* out, double c_id, double c_sl, double c_trac);
void orc_apply_lop(void* ctx, const double* in, double* out, double c_lop);
void orc_apply(void* ctx, const double* x, double* y, double alpha, double beta);
/* individual pieces (add into out), for kernel-level parity tests */
/* far field over all other spheres (excl_near != 0: also skip near-pair source spheres) */
void orc_far_traction(void* ctx, const double* in, double* out, double c, int excl_near);
void orc_far_sl(void* ctx, const double* in, double* out, double c, int excl_near);
void orc_near_correction(void* ctx, const double* in, double* out, double c_sl, double c_trac);
/* mobility solve; returns 0 converged, 1 max iterations. density3M may be NULL. */
int orc_solve_mob(void* ctx, const double* force6n, double* vel6n, double* density3m, double tol, int restart,
                  int maxit, int* iters, double* relres);
/* set number of OpenMP threads used by the oracle (<=0: library default) */
void orc_set_threads(int n);

/* near-pair rule alone: returns count, writes up to cap pairs (sorted by target, then source) */
int orc_near_pairs(int n_spheres, const double* centers, const double* radii, int cap, int* trg, int* src);

#ifdef __cplusplus
}
#endif
#endif
