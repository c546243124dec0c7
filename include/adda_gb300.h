/* adda_gb300.h - C ABI of the GB300-native DDA hot path (FFT-accelerated interaction matvec + Krylov solve).
 *
 * Plain C: pointers, sizes, status codes; no C++ or torch types. One context holds one particle lattice on one GPU
 * (device-resident interaction matrix, work buffers and solver state for up to nrhs_max right-hand sides).
 *
 * Conventions shared with the reference (ADDA 1.3b6):
 *   - complex vectors are interleaved (re,im) doubles, dipole-major [dipole][3], length 3*ndip complex per RHS
 *     (the reference's doublecomplex argvec/resultvec, src/matvec.c:128); several RHS are stacked back to back;
 *   - position[] holds (x,y,z) lattice indices of the non-void dipoles in the box, in the reference's order
 *     (z outermost, x innermost; src/make_particle.c:1984); material[] indexes the per-material tables;
 *   - cc are polarisabilities per material and component (the reference's cc[MAX_NMAT][3], src/vars.h); the
 *     library takes their square roots itself (InitCC, src/calculator.c:266-289).
 * Every entry point returns ADDA_GB300_OK (0) or a status code; adda_gb300_last_error() describes the last failure.
 * Entry points are not reentrant on one context; different contexts may be used from different threads.
 */
#ifndef ADDA_GB300_H
#define ADDA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; negative = API/runtime error, positive = solver outcome (the reference's LogError/LogWarning cases) */
#define ADDA_GB300_OK 0
#define ADDA_GB300_EINVAL (-1)      /* bad argument (the reference's LogError on inconsistent input) */
#define ADDA_GB300_ECUDA (-2)       /* CUDA runtime error or no usable GPU */
#define ADDA_GB300_ENOMEM (-3)      /* device allocation failed */
#define ADDA_GB300_ESTATE (-4)      /* call out of order (e.g. matvec before init_dmatrix) */
#define ADDA_GB300_EBREAKDOWN 1     /* Krylov breakdown (iterative.c:684,697,960) */
#define ADDA_GB300_ESTAGNATION 2    /* residual stagnated > mc iterations (iterative.c:1509) */
#define ADDA_GB300_EMAXITER 3       /* maxiter reached without convergence (iterative.c:1507, a warning there) */
#define ADDA_GB300_CHPOINT 4        /* stopped at the checkpoint time (solve_params.chp_time, the reference's -chpoint;
                                       ProgressReport, iterative.c:308-317): the state stays in the context for
                                       adda_gb300_chpoint_save; the reference's CHP_EXIT */

enum adda_gb300_shape { ADDA_SHAPE_SPHERE = 0, ADDA_SHAPE_ELLIPSOID = 1, ADDA_SHAPE_BOX = 2 };
/* polarizability prescriptions of the reference's -pol (calculator.c:170-262); nloc and nloc_av take the Gaussian
 * width Rp of -pol nloc <Rp> and are computed by adda_gb300_polarizability_nloc */
enum adda_gb300_pol {
	ADDA_POL_LDR = 0,
	ADDA_POL_CM = 1,
	ADDA_POL_RRC = 2,
	ADDA_POL_DGF = 3,
	ADDA_POL_CLDR = 4,
	ADDA_POL_FCD = 5,
	ADDA_POL_IGT_SO = 6,
	ADDA_POL_LAK = 7,
	ADDA_POL_SO = 8,
	ADDA_POL_NLOC = 9,
	ADDA_POL_NLOC_AV = 10
};
/* Krylov methods of the reference's -iter: qmr, bicgstab, bicg (BiCG_CS / COCG), cgnr, csym, qmr2 (QMR_CS_2),
 * bcgs2 (BiCGstab(2)) */
enum adda_gb300_iter {
	ADDA_ITER_QMR_CS = 0,
	ADDA_ITER_BICGSTAB = 1,
	ADDA_ITER_BICG_CS = 2,
	ADDA_ITER_CGNR = 3,
	ADDA_ITER_CSYM = 4,
	ADDA_ITER_QMR_CS_2 = 5,
	ADDA_ITER_BCGS2 = 6
};
/* arithmetic of a matvec / solve. FP64: everything in double. FP32: complex-float FFTs, D-matrix and vectors.
 * MIXED (solve only): Krylov solves whose matvec runs in FP32 (FFTs, D, expanded grid) while the Krylov vectors are
 * double-float (pairs of floats, about 48 significant bits, updated with error-free FP32 arithmetic), the
 * recurrence scalars FP64 and the reductions end in FP64, inside an iterative-refinement loop whose residual is
 * recomputed with the FP64 matvec (the reference's ResidualNorm2, iterative.c:322-338) until it meets eps.
 * MIXED_F64VEC (solve only): the same with FP64 Krylov vectors (slower on GPUs with a reduced FP64 rate).
 * MIXED_F32VEC (solve only): the same with the Krylov vectors in FP32. */
enum adda_gb300_prec {
	ADDA_PREC_FP64 = 0,
	ADDA_PREC_FP32 = 1,
	ADDA_PREC_MIXED = 2,
	ADDA_PREC_MIXED_F32VEC = 3,
	ADDA_PREC_MIXED_F64VEC = 4
};
/* interaction terms of the reference's -int (interaction.c:290-411,431-941): point dipoles, filtered coupled dipoles
 * (FCD, Gay-Balmaz & Martin / Piller) and its static limit, the static non-local interaction of two Gaussian
 * dipole densities of width Rp (problem.nloc_rp; nloc: point value of the non-locality function, nloc_av: its average
 * over the dipole cube), and the two terms built on the reference's tabulated integrals of the Green's tensor over
 * the dipole cube (problem.int_tables): the approximate integrated Green's tensor igt_so (InterTerm_igt_so_int) and
 * the second-order formulation so (InterTerm_so_int, in the reference's orientation-averaged form; its m^2 terms use
 * problem.so_m). igt (a cubature per lattice offset) is not provided. */
enum adda_gb300_inter { ADDA_INT_POI = 0, ADDA_INT_FCD = 1, ADDA_INT_FCD_ST = 2, ADDA_INT_NLOC = 3,
	ADDA_INT_NLOC_AV = 4, ADDA_INT_IGT_SO = 5, ADDA_INT_SO = 6 };
/* the integral tables of igt_so and so: the reference's input/tables/t1f.dat .. t10f.dat back to back (142 entries of
 * 1, 6, 3, 18, 6, 36, 1, 6, 1, 6 values each: 11928 doubles; ReadTables, interaction.c:1031-1063) */
#define ADDA_GB300_INT_TABLES 11928
/* -init_field: auto, zero, inc (CalcInitField, iterative.c:1342-1394), and X0: the starting vector x_0 is supplied by
 * the caller in xvec (host API) or d_xvec (device API) -- the reference's "read" and "wkb" modes, which turn an
 * electric field E into x_0 = E/(cc_sqrt*chi_inv) (InitFieldfromE, iterative.c:1325-1338; see
 * adda_gb300_wkb_field) */
enum adda_gb300_init_field { ADDA_IF_AUTO = 0, ADDA_IF_ZERO = 1, ADDA_IF_INC = 2, ADDA_IF_X0 = 3, ADDA_IF_CHPOINT = 4 };
/* ADDA_IF_CHPOINT: every right-hand side resumes from the state given to adda_gb300_chpoint_load (the reference's
 * -chp_load, LoadIterChpoint, iterative.c:222-278); FP64 only */

/* reflected Green's tensor of a particle near a substrate (-int_surf, interaction.c:1082-1345):
 * IMG  image-dipole approximation, computed on the GPU (ReflTerm_img);
 * SOM  image dipole plus the Sommerfeld-integral correction; refl_data holds the four integrals Irv, Izv, Irh, Iph
 *      (complex) for every in-plane offset (i < boxX, j < boxY) and height sum k < 2*boxZ-1, layout [k][j][i][4],
 *      evaluated at rho = hypot(i,j)*d, z = (k + zsum_shift)*d (the table of CalcSomTable, interaction.c:1176-1224,
 *      on the full rectangle); they are combined with the image term on the GPU (ReflTerm_som_int);
 * HOST the reflected tensor itself from the caller (e.g. the reference's own ReflTerm_int): refl_data [k][j][i'][6]
 *      complex for k < 2*boxZ-1, j < boxY, i' = i + boxX - 1 < 2*boxX-1 (components xx,xy,xz,yy,yz,zz). */
enum adda_gb300_refl { ADDA_REFL_IMG = 0, ADDA_REFL_SOM = 1, ADDA_REFL_HOST = 2 };

typedef struct adda_gb300_ctx adda_gb300_ctx;

/* The particle lattice: replaces the globals the reference sets in ParSetup/MakeParticle (comm.c:481-535,
 * make_particle.c:2185-2230) and reads in InitDmatrix/MatVec. */
typedef struct {
	int boxX, boxY, boxZ;        /* computational box; boxX,boxY,boxZ >= 1 */
	int gridX, gridY, gridZ;     /* padded FFT grid; 0 = fftFit(2*box) as ParSetup does (comm.c:489-491) */
	size_t ndip;                 /* non-void dipoles */
	const uint16_t *position;    /* [ndip][3], sorted z-major then y then x (the reference's order) */
	const uint8_t *material;     /* [ndip] material index, or NULL (all 0) */
	double gridspace;            /* lattice spacing d (lambda/dpl) */
	double wavenum;              /* k = 2*pi/lambda */
	int nrhs_max;                /* right-hand sides solved together (>=1) */
	int device;                  /* CUDA device ordinal */
	int interaction;             /* enum adda_gb300_inter (-int); 0 = point dipoles */
	double nloc_rp;              /* Gaussian width Rp of -int nloc|nloc_av <Rp> (same length unit as gridspace) */
	/* particle near a substrate (-surf <h> <m_re> <m_im> | -surf <h> inf); all ignored when surface == 0 */
	int surface;
	double zsum_shift;           /* ZsumShift (make_particle.c:2309): 2*(h/d - (boxZ-1)/2), in lattice units; the
	                                lowest dipole layer zmin must be above the substrate: zsum_shift + 2*zmin > 0 */
	double msub_re, msub_im;     /* substrate refractive index */
	int msub_inf;                /* perfectly reflecting substrate (reflection coefficient -1, image relation) */
	int refl;                    /* enum adda_gb300_refl */
	const double *refl_data;     /* SOM / HOST data (copied by adda_gb300_create), NULL for IMG */
	/* interaction IGT_SO / SO: the integral tables (ADDA_GB300_INT_TABLES doubles, see adda_gb300_read_int_tables;
	 * copied by adda_gb300_create), and SO's refractive index (the reference's ref_index[0]) */
	const double *int_tables;
	double so_m_re, so_m_im;
} adda_gb300_problem;

typedef struct {
	int method;                  /* enum adda_gb300_iter (-iter) */
	int precision;               /* ADDA_PREC_FP64, ADDA_PREC_MIXED, ADDA_PREC_MIXED_F64VEC or ADDA_PREC_MIXED_F32VEC */
	double eps;                  /* relative residual target (-eps e => 10^-e) */
	int maxiter;                 /* -maxiter */
	int init_field;              /* enum adda_gb300_init_field (-init_field) */
	int check_every;             /* iterations between host convergence checks (CUDA graph length); 0 = default */
	double inner_eps;            /* MIXED: relative tolerance of each FP32 inner solve; 0 = default */
	int max_refine;              /* MIXED: maximum outer refinement steps; 0 = default */
	double chp_time;             /* FP64: > 0 stops the solve once this many seconds of wall time have passed (checked
	                                every check_every iterations) with status ADDA_GB300_CHPOINT for the right-hand
	                                sides still running (-chpoint <time>); 0 = none */
	int full_steps;              /* BiCGStab: no exit at the half step (the reference with -chp_type always,
	                                iterative.c:703), so that the final state is a complete iteration */
	double final_eps;            /* MIXED: FP64 relative residual at which the refinement loop stops, 0 < final_eps
	                                <= eps; 0 = the default, 0.3*eps (0.1*eps for BiCGStab, BCGS2 and FP32 Krylov
	                                vectors, ADDA_PREC_MIXED_F32VEC). The solve
	                                succeeds once the residual meets eps; the margin below eps makes the cross
	                                sections as accurate as a converged FP64 solve's to about 1e-6, which a solution
	                                that only just meets a residual of 1e-5 is not (on the 128^3 sphere the FP64
	                                solve at eps 1e-5 is 6e-6 off the converged Cabs, and the reference's own run
	                                too) */
} adda_gb300_solve_params;

typedef struct {
	int niter;                   /* Krylov iterations (reference: IterativeSolver's return value) */
	int status;                  /* ADDA_GB300_OK or solver outcome code */
	double resid;                /* final relative residual; MIXED: the FP64 recomputed one */
	int refinements;             /* MIXED: outer steps; FP64: 0 */
	int matvecs_fp64, matvecs_fp32;
} adda_gb300_rhs_stats;

/* ---- particle-side inputs (host code, no GPU) --------------------------------------------------------------- */

/* ReadTables / ReadTableFile, src/interaction.c:1004-1063: the ten files t1f.dat .. t10f.dat of directory dir (the
 * reference's input/tables) into tables[ADDA_GB300_INT_TABLES]; EINVAL when a file is missing or too short */
int adda_gb300_read_int_tables(const char *dir, double *tables);

/* fftFit, src/fft.c:528-562: smallest even size >= x, divisible by divis, with prime factors 2,3,5,7 (+ one 11|13) */
int adda_gb300_fft_fit(int x, int divis);
/* boxY/boxZ from boxX and the shape's aspect ratios: InitShape sizing, src/make_particle.c:1283-1308,1912-1919.
 * pars: ellipsoid/box aspect ratios (y/x, z/x), or NULL for a sphere/cube. */
int adda_gb300_fit_box(int shape, const double *pars, int boxX, int *boxY, int *boxZ);
/* MakeParticle's box loop, src/make_particle.c:1984-2230. Returns ndip; position/material may be NULL to count. */
size_t adda_gb300_make_particle(int shape, const double *pars, int boxX, int boxY, int boxZ, uint16_t *position,
	uint8_t *material);
/* Incident frame: propagation prop0 (NULL = (0,0,1); -prop, param.c:1371-1382) with its two polarisations
 * (param.c:2116-2131), rotated by the zyz Euler angles in degrees (-orient; InitRotation, src/crosssec.c:82-139) */
void adda_gb300_rotation(const double prop0[3], double alpha_deg, double beta_deg, double gamma_deg, double prop[3],
	double incPolY[3], double incPolX[3]);
/* GenerateB, free-space plane wave, src/GenerateB.c:324-328: einc[i] = pol * exp(i k r_i.prop) */
void adda_gb300_plane_wave(size_t ndip, const uint16_t *position, int boxX, int boxY, int boxZ, double gridspace,
	double wavenum, const double prop[3], const double pol[3], double *einc);
/* GenerateB, plane wave for a particle whose centre is hsub above a substrate of index msub (msub_inf: perfectly
 * reflecting), src/GenerateB.c:96-140, 257-323. which: 0 = the Y polarisation (s), 1 = X (p). From above (prop[2] <
 * 0) the incident plus the Fresnel-reflected wave; from below (prop[2] > 0, finite msub only) the transmitted wave.
 * inc_scale receives the cross-section factor (1/Re(msub) from below, else 1). EINVAL for prop[2] == 0. */
int adda_gb300_plane_wave_surf(size_t ndip, const uint16_t *position, int boxX, int boxY, int boxZ,
	double gridspace, double wavenum, const double prop[3], const double incPolY[3], const double incPolX[3],
	int which, double hsub, double msub_re, double msub_im, int msub_inf, double *einc, double *inc_scale);

/* CalcFieldWKB (iterative.c:1227-1322): the internal field in the WKB approximation for incidence along +z:
 * E_j = Einc_j exp(phi_j), phi accumulated along each z column of the box with i(m-1)kd/2 per half cell (void cells
 * add nothing). material [ndip] (NULL = all 0), ref_index [nmat][2] (re, im); einc and field [ndip][3] complex. */
int adda_gb300_wkb_field(int boxX, int boxY, int boxZ, size_t ndip, const uint16_t *position, const uint8_t *material,
	int nmat, const double *ref_index, double kd, const double *einc, double *field);
/* CoupleConstant, src/calculator.c:170-262 (enum adda_gb300_pol; LDR with avgpol); cc = the 3 diagonal components
 * (identical except for CLDR) */
int adda_gb300_polarizability(int relation, double m_re, double m_im, double kd, double gridspace,
	const double prop[3], const double incPol[3], int avgpol, double cc[6]);

/* -pol nloc|nloc_av <Rp> (calculator.c:223-248, static): M = (4pi/3) ellTheta(d/(sqrt(2pi) Rp)) for nloc (lattice sum
 * of the Gaussian's non-locality function) and (4pi/3)(1 - erf(d/(2 sqrt(2) Rp))^3) for nloc_av; Rp = 0 gives CM */
int adda_gb300_polarizability_nloc(int relation, double m_re, double m_im, double gridspace, double rp, double cc[6]);

/* d(1/alpha)/dchi for the same relations (chi = (m^2-1)/(4pi), the susceptibility), the input of adda_gb300_vjp_chi */
int adda_gb300_polarizability_dchi(int relation, double m_re, double m_im, double kd, double gridspace,
	const double prop[3], const double incPol[3], int avgpol, double out[2]);

/* ---- device context ------------------------------------------------------------------------------------------ */

/* ParSetup + allocation half of InitDmatrix (comm.c:481-535, fft.c:1164-1209): validates the lattice, uploads it
 * and allocates every device buffer. Fails with ADDA_GB300_ECUDA when no GPU is usable. */
int adda_gb300_create(const adda_gb300_problem *p, adda_gb300_ctx **out);
/* Several particles solved as one batch (no counterpart in the reference, which solves particles one after another,
 * calculator.c:348-358): nparticles lattices of ndip[q] dipoles (positions[q], materials[q] or NULL) in the common box
 * and grid of p (every particle inside it; p->ndip, p->position and p->material are ignored), sharing D; p->nrhs_max
 * = nparticles x the RHS per particle, and RHS r belongs to particle r / (nrhs_max / nparticles). Vectors have the
 * largest particle's length ndip_max per RHS, [nrhs][ndip_max][3]: the entries past a smaller particle's ndip[q] are
 * padding, which the incident field must leave at zero and the solve keeps at zero (adda_gb300_matvec returns zeros
 * there, adda_gb300_matvec_device leaves the padding of d_res as it was); set_cc per RHS gives each
 * particle its own polarizabilities. The phase reference of the incident field, the cross sections and the scattered
 * fields is the centre of the common box (a particle's own box centre only shifts the phase of its solution). Every matvec stage, vector update and reduction then runs once for all
 * particles' RHS (one launch per stage, one CUDA graph per batch of iterations), and a particle whose RHS have all
 * converged costs no more FFT work. Free space only; checkpoints and the VJP take single-lattice contexts. */
int adda_gb300_create_group(const adda_gb300_problem *p, int nparticles, const size_t *ndip,
	const uint16_t *const *positions, const uint8_t *const *materials, adda_gb300_ctx **out);
/* Free_FFT_Dmat, src/fft.c:1420-1493 */
int adda_gb300_destroy(adda_gb300_ctx *ctx);
/* grid actually used (after fftFit) */
int adda_gb300_get_grid(const adda_gb300_ctx *ctx, int grid[3]);

/* InitDmatrix, src/fft.c:918-1416: Green's tensor (point dipoles, interaction.c:290-331) and its FFT, computed in
 * FP64 on the GPU, kept in the reduced (y<=gY/2, z<=gZ/2) layout plus an FP32 copy. */
int adda_gb300_init_dmatrix(adda_gb300_ctx *ctx);
/* copy the FP64 D matrix to the host: layout [x][z<gZ/2+1][y<gY/2+1][6] complex (fft.c:144-150) */
size_t adda_gb300_dmatrix_len(const adda_gb300_ctx *ctx);
int adda_gb300_get_dmatrix(adda_gb300_ctx *ctx, double *out);
/* surface mode: InitRmatrix, src/fft.c:818-887, built with D by adda_gb300_init_dmatrix: R = -FFT(GR)/Ngrid with the
 * height sums along z, reduced in y only; copy of the FP64 R: layout [x][z<gZ][y<gY/2+1][6] complex (fft.c:196-201);
 * length 0 without a substrate */
size_t adda_gb300_rmatrix_len(const adda_gb300_ctx *ctx);
int adda_gb300_get_rmatrix(adda_gb300_ctx *ctx, double *out);

/* InitCC, src/calculator.c:266-289, for right-hand side rhs: cc per material [nmat][3] complex */
int adda_gb300_set_cc(adda_gb300_ctx *ctx, int rhs, int nmat, const double *cc);
/* same with the square roots given directly (the reference's cc_sqrt[MAX_NMAT][3] after InitCC); cc = cc_sqrt^2 is
 * kept for the absorption cross section */
int adda_gb300_set_cc_sqrt(adda_gb300_ctx *ctx, int rhs, int nmat, const double *cc_sqrt);
/* per-dipole polarisabilities [ndip][3] complex for right-hand side rhs (inhomogeneous media) */
int adda_gb300_set_cc_dipole(adda_gb300_ctx *ctx, int rhs, const double *cc);

/* MatVec, src/matvec.c:128-425, for nrhs stacked vectors in HOST memory: resultvec = argvec + S.D.S.argvec,
 * S = diag(sqrt(cc)); her != 0 applies the Hermitian transpose; inprod (may be NULL) receives |resultvec_r|^2 per
 * RHS. prec = ADDA_PREC_FP64 or ADDA_PREC_FP32 (the FP32 path rounds the inputs to complex float). */
int adda_gb300_matvec(adda_gb300_ctx *ctx, int prec, int nrhs, const double *argvec, double *resultvec,
	double *inprod, int her);
/* same, on DEVICE buffers (double2 for FP64, float2 for FP32) on the context's stream; no host synchronisation.
 * The call starts after the work queued before it on the caller's stream (adda_gb300_set_stream) and work queued on
 * that stream after the call runs after the results are written. */
int adda_gb300_matvec_device(adda_gb300_ctx *ctx, int prec, int nrhs, const void *d_argvec, void *d_resultvec,
	double *d_inprod, int her);

/* IterativeSolver, src/iterative.c:1398-1530, for nrhs right-hand sides at once. einc: incident fields
 * [nrhs][ndip][3] (host). On return xvec (may be NULL) holds the solution x and pvec (may be NULL) the polarisations
 * S.x; both also stay on the device for adda_gb300_cross_sections. stats: one entry per RHS (may be NULL).
 * resid_hist (may be NULL): [nrhs][hist_cap] relative residuals RE_000, RE_001, ... (iterative.c:69,301). */
int adda_gb300_solve(adda_gb300_ctx *ctx, const adda_gb300_solve_params *sp, int nrhs, const double *einc,
	double *xvec, double *pvec, adda_gb300_rhs_stats *stats, double *resid_hist, int hist_cap);

/* Iteration checkpoints in the reference's chp.<ringid> byte format (SaveIterChpoint / LoadIterChpoint,
 * src/iterative.c:165-278; native byte order, the reference's layout: int ind_m, size_t local_nRows, int niter, int
 * counter, double inprodR, prev_err, resid_scale, the method's scalars, xvec, rvec, pvec, the method's vectors), so
 * that a state saved by the reference resumes here and vice versa.
 * adda_gb300_chpoint_size: bytes of a checkpoint of the given method for this lattice.
 * adda_gb300_chpoint_save: the state of right-hand side rhs after the last FP64 solve (finished, or stopped with
 * ADDA_GB300_CHPOINT) into buf (size >= adda_gb300_chpoint_size); ADDA_GB300_ESTATE when there is none (no FP64
 * solve yet, a later MIXED solve or matvec-only use, or a breakdown).
 * adda_gb300_chpoint_load: checks and keeps a checkpoint for right-hand side rhs until the next solve with
 * init_field ADDA_IF_CHPOINT; ADDA_GB300_EINVAL for a file of another size or vector length (the reference's
 * "different vector size" / "too long" / "Failed reading" errors, iterative.c:238-266). The method is checked by the
 * solve ("different iterative method"). */
size_t adda_gb300_chpoint_size(const adda_gb300_ctx *ctx, int method);
int adda_gb300_chpoint_save(adda_gb300_ctx *ctx, int rhs, void *buf, size_t size);
int adda_gb300_chpoint_load(adda_gb300_ctx *ctx, int rhs, const void *buf, size_t size);

/* same as adda_gb300_solve with DEVICE buffers (double2 [nrhs][ndip][3]) for einc and the optional d_xvec/d_pvec:
 * nothing crosses PCIe/C2C except the per-RHS stats and the convergence flags polled between graph launches. The
 * solve reads d_einc and d_xvec after the work queued before the call on the caller's stream (adda_gb300_set_stream)
 * and returns when d_xvec and d_pvec are written. */
int adda_gb300_solve_device(adda_gb300_ctx *ctx, const adda_gb300_solve_params *sp, int nrhs, const void *d_einc,
	void *d_xvec, void *d_pvec, adda_gb300_rhs_stats *stats);

/* The caller's stream for the device-buffer calls (adda_gb300_matvec_device, adda_gb300_solve_device): a cudaStream_t
 * of the context's device, or NULL for the legacy default stream (the default). The context computes on streams of
 * its own that do not synchronise with other streams, so buffers a caller fills on a stream must be ordered before
 * the call through this stream (or be complete: e.g. after a cudaStreamSynchronize). */
int adda_gb300_set_stream(adda_gb300_ctx *ctx, void *stream);

/* Several particles at once (uneven grids): solves context i for nrhs[i] right-hand sides einc[i] (host), writing
 * xvec[i]/pvec[i] (host, may be NULL) and stats[i] (nrhs[i] entries, may be NULL). The contexts run concurrently, each
 * on its own stream from its own host thread, so small lattices share the GPU instead of queueing. Returns the first
 * non-zero status (and keeps going for the others). The reference solves particles one after another
 * (orientation/particle loops of calculator.c:348-358 around IterativeSolver). */
int adda_gb300_solve_many(int nctx, adda_gb300_ctx *const *ctxs, const adda_gb300_solve_params *sp, const int *nrhs,
	const double *const *einc, double *const *xvec, double *const *pvec, adda_gb300_rhs_stats *const *stats);

/* ExtCross (plane wave) and AbsCross (Draine), src/crosssec.c:811-917, in FP64 on the device from the
 * polarisations left by the last solve: prop/incpol per RHS [nrhs][3]; cext/cabs per RHS. */
int adda_gb300_cross_sections(adda_gb300_ctx *ctx, int nrhs, const double *prop, const double *incpol,
	double *cext, double *cabs);
/* ExtCross for a general incident field, the branch the reference takes in surface mode (src/crosssec.c:823-846):
 * Cext = 4 pi k sum_j Im(P_j . conj(Einc_j)) * inc_scale, and AbsCross * inc_scale (inc_scale from
 * adda_gb300_plane_wave_surf), from the polarisations of the last solve; einc [nrhs][ndip][3] complex (host). */
int adda_gb300_cross_sections_beam(adda_gb300_ctx *ctx, int nrhs, const double *einc, double inc_scale,
	double *cext, double *cabs);

/* ---- integrals over scattering directions (host code; fields from the GPU) ------------------------------------- */

/* one block of the reference's alldir_params.dat (theta: equal steps in cos, phi: equal steps in the angle; degrees):
 * ScanIntegrParms, src/crosssec.c:233-307. The reference's defaults are theta {0, 180, 2, 6, 0, 0, 0} and phi
 * {0, 360, 2, 5, 0, 1, 1}. */
typedef struct {
	double min, max;   /* degrees */
	int Jmin, Jmax;    /* refinement stages: 2^Jmax + 1 grid points */
	double eps;        /* relative error at which the integration may stop; 0 = use every point */
	int equiv;         /* min and max are the same direction: the last point is not stored */
	int periodic;      /* trapezoid rule instead of Romberg extrapolation */
} adda_gb300_integr_parms;

/* the grid angles in degrees (val may be NULL): equal steps in cos(angle) for in_cos (theta, from max down to min),
 * in the angle otherwise. Returns the number of points, -1 for parameters the reference rejects. */
int adda_gb300_integr_points(const adda_gb300_integr_parms *p, int in_cos, double *val);
/* Romberg2D (src/Romberg.c:175-533): average over theta (outer, p[0]) and phi (inner, p[1]) of values
 * [ntheta][nphi][dim] given on the grids above; returns the relative error estimate (-1 for bad arguments) */
double adda_gb300_romberg2d(const adda_gb300_integr_parms p[2], int dim, const double *values, double *res);
/* the same with poles != 0 for orientation averaging over the full range of the first Euler angle (full_al_range,
 * src/crosssec.c:369): at beta = 180 and beta = 0 every gamma is the same orientation, so the inner integral there is
 * the value at gamma index 0 (OuterInitT's onepoint, src/Romberg.c:374-386) */
double adda_gb300_romberg2d_ex(const adda_gb300_integr_parms p[2], int dim, const double *values, double *res,
	int poles);
/* Csca and Csca*g of each RHS r < nrhs from the last solve (CalcAlldir + ScaCross + AsymParm_x/y/z, free space,
 * src/crosssec.c:991-1260): the scattered field on the grid of p (directions cos(theta) prop + sin(theta)
 * (cos(phi) incPolX + sin(phi) incPolY), SetScatPlane :944-990) on the GPU, |E|^2 and the Romberg integrals on the
 * host. csca [nrhs]; csca_g [nrhs][3] in the beam frame (incPolX, incPolY, prop), g = csca_g / csca. */
int adda_gb300_scattering_integrals(adda_gb300_ctx *ctx, int nrhs, const adda_gb300_integr_parms p[2],
	const double prop[3], const double incpolx[3], const double incpoly[3], double *csca, double *csca_g);

/* Scattering amplitudes, CalcField / CalcFieldFree (src/crosssec.c:506-596, 801-808; free space, Draine
 * scattering relation), in FP64 on the device from the polarisations left by the last solve:
 * E_r(n) = (-i k^3) exp(-i k r0.n) (I - nn).sum_j P_rj exp(-i kd n.pos_j) for each RHS r < nrhs and each unit
 * direction n of dirs [ndir][3]; ebuff [nrhs][ndir][3] complex (interleaved re, im). The reference's callers
 * (CalcEplaneYZ and friends, CalculateE.c:423-500) turn these into Mueller matrices; so does the Python layer. */
int adda_gb300_scattered_fields(adda_gb300_ctx *ctx, int nrhs, int ndir, const double *dirs, double *ebuff);

/* average device time of one matvec (prec, nrhs RHS, device-resident random input) over iters launches, measured
 * with CUDA events on the context's stream after one warm-up launch; flush_bytes > 0 writes that many bytes of a
 * scratch buffer between launches so every launch starts with a cold L2 */
int adda_gb300_time_matvec(adda_gb300_ctx *ctx, int prec, int nrhs, int iters, size_t flush_bytes, double *ms);

/* The matvec's tile shape for one arithmetic (prec ADDA_PREC_FP64 or ADDA_PREC_FP32): shape[0] y-lines per block of
 * the scatter + x-FFT and inverse x-FFT + gather kernels, [1] y-lines per block of the z-FFT kernels, [2] (kz, RHS)
 * pairs per block of the generic y-FFT + D kernel, [3] threads per block of the register y-FFT + D kernel (FP32).
 * The library picks the defaults, narrows them for axes longer than 512 (up to 2048 per axis), and tunes the FP32
 * shape at the first FP32 matvec or solve of a context together with its L2 chunk (the reference plans its FFTs
 * with FFTW_MEASURE likewise, fft.c:739-815). No counterpart call in the reference: its FFTs are FFTW's. */
int adda_gb300_get_fft_shape(const adda_gb300_ctx *ctx, int prec, int shape[4]);
/* x-slabs per chunk of the y/z stage (the L2 chunk; FP32: tuned with the shape), or EINVAL */
int adda_gb300_get_l2_chunk(const adda_gb300_ctx *ctx, int prec);
/* set a shape (FP32: the tuner then keeps it; the L2 chunk is still tuned); EINVAL for a shape this build does not
 * hold for the context's axis lengths or one whose shared memory does not fit a block. The environment variable
 * ADDA_GB300_FFT_SHAPE="w1,w2,pairs,threads" does the same for every FP32 context. */
int adda_gb300_set_fft_shape(adda_gb300_ctx *ctx, int prec, const int shape[4]);

/* device time in milliseconds of the last solve on this context: CUDA events recorded on the context's stream at
 * the first and the last kernel of the solve (host-device copies of the host-pointer API excluded) */
double adda_gb300_last_solve_ms(const adda_gb300_ctx *ctx);

/* Adjoint (VJP) of Cext and Cabs of right-hand side `rhs` of the last solve with respect to every dipole's
 * susceptibility chi_j (isotropic), by one more solve with the same complex-symmetric matrix (A^T = A), for the two
 * adjoint right-hand sides at once: extinction (Cext is linear in P, crosssec.c:811-822) and absorption (Cabs is
 * quadratic in P and depends on alpha, crosssec.c:866-882). dinv_alpha [ndip] complex = d(1/alpha_j)/dchi_j (see
 * adda_gb300_polarizability_dchi). Outputs [ndip][2]: (dC/dRe chi_j, dC/dIm chi_j). sp selects the arithmetic of the
 * adjoint solve. Requires nrhs_max >= 2; the forward polarisations stay available for adda_gb300_cross_sections. */
int adda_gb300_vjp_chi(adda_gb300_ctx *ctx, const adda_gb300_solve_params *sp, int rhs, const double prop[3],
	const double incpol[3], const double *dinv_alpha, double *grad_cext, double *grad_cabs);

/* Allocation-free variant of adda_gb300_cross_sections; it has no counterpart in the reference (whose host never
 * runs where allocation is forbidden). For callers that cannot call cudaMalloc at this point: code running inside a
 * framework that owns all device memory through its own pool allocator, or a plugin whose host forbids device
 * allocation after start-up. Free space only (plane-wave ExtCross and AbsCross, crosssec.c:811-822,866-882): for a
 * particle near a substrate use adda_gb300_cross_sections_beam.
 * Everything is passed as device pointers: polarisations d_pvec [nrhs][ndip][3] double2, d_position [ndip][3],
 * d_material [ndip] (or NULL for one material; every index must be below nmat, else that RHS's Cabs is NaN),
 * polarisabilities d_cc [nrhs][nmat][3] (per_dipole=0) or [nrhs][ndip][3] (per_dipole=1) double2,
 * d_prop/d_incpol [nrhs][3]; results to d_cext/d_cabs [nrhs]. The call is asynchronous on `stream` (a cudaStream_t,
 * or NULL) and allocates nothing: its partial sums live in a 1 MiB static device array (256 partials x 8 doubles x
 * ADDA_GB300_NOALLOC_MAX_RHS) that every GPU loading the library holds until exit. The first call on a device looks
 * up that array's address (make it before any stream capture). All calls share the array: calls that overlap on the
 * GPU race. nrhs > ADDA_GB300_NOALLOC_MAX_RHS is rejected (ADDA_GB300_EINVAL). */
#define ADDA_GB300_NOALLOC_MAX_RHS 64
int adda_gb300_cross_sections_noalloc(int nrhs, size_t ndip, const void *d_pvec, const uint16_t *d_position,
	const uint8_t *d_material, const void *d_cc, int nmat, int per_dipole, int boxX, int boxY, int boxZ,
	double gridspace, double wavenum, const double *d_prop, const double *d_incpol, double *d_cext, double *d_cabs,
	void *stream);

/* last error message of the calling thread */
const char *adda_gb300_last_error(void);
/* number of kernels this library has launched in the calling process (for launch accounting) */
uint64_t adda_gb300_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif
