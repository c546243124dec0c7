/* adda_oracle.h - CPU restatement of ADDA's FFT-accelerated DDA hot path (double precision).
 *
 * TEST INFRASTRUCTURE (oracle). Used only by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg,
 * always as the checker or the timed CPU baseline, never as part of the GPU product.
 *
 * What is restated (reference = ADDA 1.3b6, paths relative to the reference project):
 *   or_init_dmatrix  <- InitDmatrix              src/fft.c:918-1416 (reduced FFT) with the interaction terms
 *                                               InterTerm_poi/fcd/fcd_st/nloc/nloc_av/igt_so/so
 *                                               (src/interaction.c:290-941)
 *   or_matvec        <- MatVec                   src/matvec.c:128-425
 *   or_solve         <- IterativeSolver          src/iterative.c:1398-1530, QMR_CS :898-1032, BiCGStab :640-724,
 *                                               BiCG_CS :490-637, CGNR :729-769, CSYM :773-892,
 *                                               QMR_CS_2 :1038-1132, BCGS2 :340-487
 *   or_solve_chp     <- SaveIterChpoint / LoadIterChpoint  src/iterative.c:165-278
 *   or_cross         <- ExtCross / AbsCross      src/crosssec.c:811-917 (plane wave, free space, Draine)
 *   or_field         <- CalcFieldFree            src/crosssec.c:506-596 (scattering amplitude in one direction)
 *   or_set_surface   <- particle near a substrate: ReflTerm_img / ReflTerm_som (src/interaction.c:1082-1345),
 *                       InitRmatrix (src/fft.c:818-887), the reflected part of MatVec (src/matvec.c:249-303)
 *   or_cross_beam    <- ExtCross for a general incident field (src/crosssec.c:823-845), AbsCross
 * Complex vectors are interleaved (re,im) doubles, dipole-major [dipole][3], like the reference's doublecomplex.
 */
#ifndef ADDA_ORACLE_H
#define ADDA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

typedef struct or_ctx or_ctx;

/* iterative methods and initial-field modes, same meaning as -iter and -init_field */
enum { OR_QMR_CS = 0, OR_BICGSTAB = 1, OR_BICG_CS = 2, OR_CGNR = 3, OR_CSYM = 4, OR_QMR_CS_2 = 5, OR_BCGS2 = 6 };
enum { OR_IF_AUTO = 0, OR_IF_ZERO = 1, OR_IF_INC = 2, OR_IF_X0 = 3 }; /* X0: x_0 given in xvec */
/* solver status codes */
enum { OR_OK = 0, OR_EBREAKDOWN = 1, OR_ESTAGNATION = 2, OR_EMAXITER = 3 };

int or_fftfit(int x, int divis);
or_ctx *or_create(int boxX, int boxY, int boxZ, int gridX, int gridY, int gridZ, size_t nvoid,
	const uint16_t *position, const uint8_t *material, double gridspace, double wavenum, int nthreads);
void or_free(or_ctx *c);
/* interaction term of D: 0 point dipoles (InterTerm_poi), 1 FCD (InterTerm_fcd), 2 static FCD (InterTerm_fcd_st),
 * src/interaction.c:315-411; set before or_init_dmatrix */
void or_set_interaction(or_ctx *c, int relation);
/* 3 = -int nloc, 4 = -int nloc_av (src/interaction.c:589-707): their Gaussian width Rp (gridspace units) */
void or_set_nloc_rp(or_ctx *c, double rp);
/* 5 = -int igt_so, 6 = -int so (src/interaction.c:431-579, 711-941): the reference's integral tables t1f..t10f.dat
 * (ReadTables, src/interaction.c:1031-1063; TAB_SIZE 142 entries of 1,6,3,18,6,36,1,6,1,6 values each, src/const.h:276)
 * back to back, and for SO the refractive index of its second-order terms (ref_index[0]); set before
 * or_init_dmatrix */
#define OR_TAB_RMAX 10
#define OR_TAB_SIZE 142
#define OR_TAB_TOTAL (OR_TAB_SIZE * 84)
void or_set_tables(or_ctx *c, const double *tables, double m_re, double m_im);
/* cosine and sine integrals Ci(x), Si(x) for x > 0 (the reference's cisi, sinint.c) */
void or_cisi(double x, double *ci, double *si);
void or_init_dmatrix(or_ctx *c);
size_t or_dmatrix_len(const or_ctx *c);        // complex elements, layout [x][z<DsizeZ][y<DsizeY][6]
void or_get_dmatrix(const or_ctx *c, double *out);
/* coupling constants: cc (not its root) per material [nmat][3] or per dipole [N][3]; cc_sqrt=csqrt(cc) */
void or_set_cc_mat(or_ctx *c, int nmat, const double *cc);
void or_set_cc_dip(or_ctx *c, const double *cc);
void or_matvec(or_ctx *c, const double *argvec, double *resultvec, double *inprod, int her);
int or_solve(or_ctx *c, int method, const double *einc, double eps, int maxiter, int init_field,
	double *xvec, double *pvec, double *resid_hist, int hist_cap, int *niter_out);
/* or_solve with the reference's iteration checkpoints (SaveIterChpoint / LoadIterChpoint, src/iterative.c:165-278):
 * chp_in (chp_in_len bytes, the reference's chp.<ringid> format) replaces the initialisation by the saved state
 * (the residual history then starts at the saved iteration number, resid_hist[0] = its RE value); chp_out receives
 * the state at the end of the solve like -chp_type always (iterative.c:1498), *chp_out_len = bytes needed (written
 * only when they fit the capacity passed in *chp_out_len). Returns -1 for a checkpoint of another method or size. */
int or_solve_chp(or_ctx *c, int method, const double *einc, double eps, int maxiter, int init_field,
	double *xvec, double *pvec, double *resid_hist, int hist_cap, int *niter_out, const void *chp_in,
	size_t chp_in_len, void *chp_out, size_t *chp_out_len);
void or_cross(or_ctx *c, const double *pvec, const double prop[3], const double incpol[3], double *cext,
	double *cabs);
void or_field(const or_ctx *c, const double *pvec, const double n[3], double *ebuff);
/* surface mode, set before or_init_dmatrix (which then also builds R): ZsumShift (lattice units), the substrate's
 * refractive index (msub_inf: perfectly reflecting), and the Sommerfeld integrals Irv, Izv, Irh, Iph per
 * (k < 2bZ-1, j < bY, i < bX) at rho = hypot(i,j) d, z = (k + ZsumShift) d (NULL: image-dipole relation) */
void or_set_surface(or_ctx *c, double zsum_shift, double msub_re, double msub_im, int msub_inf,
	const double *som_table);
size_t or_rmatrix_len(const or_ctx *c);        // complex elements, layout [x][z<gridZ][y<gridY/2+1][6]
void or_get_rmatrix(const or_ctx *c, double *out);
void or_cross_beam(or_ctx *c, const double *pvec, const double *einc, double inc_scale, double *cext, double *cabs);

#endif
