/* adda_dropin.h - the reference's own entry points of the FFT matvec path, as exported by the drop-in object
 * adda_dropin.o (a-dda_gb300/csrc/dropin/adda_dropin.c) on top of libadda_gb300.
 *
 * Linking adda_dropin.o + libadda_gb300.so in place of the reference's fft.c, matvec.c and iterative.c gives the
 * unmodified ADDA host a GPU build, the same way the reference swaps matvec.c for oclmatvec.c in its OpenCL variant
 * (src/ocl/Makefile, src/seq/Makefile:19). Signatures are the reference's; the types below are the reference's
 * sequential-build types (src/types.h:30 doublecomplex, src/timing.h:29 TIME_TYPE, src/const.h:251-272 enums).
 */
#ifndef ADDA_DROPIN_H
#define ADDA_DROPIN_H

#include <complex.h>
#include <stdbool.h>
#include <time.h>

#ifndef ADDA_DROPIN_TYPES
#define ADDA_DROPIN_TYPES
typedef double complex doublecomplex;
enum iter { IT_BCGS2, IT_BICG_CS, IT_BICGSTAB, IT_CGNR, IT_CSYM, IT_QMR_CS, IT_QMR_CS_2 };
enum incpol { INCPOL_Y, INCPOL_X };
enum scat { SQ_DRAINE, SQ_FINDIP, SQ_IGT_SO, SQ_SO }; /* src/const.h:203-209 */
#endif

/* fftFit, src/fft.c:528 (fft.h:41): padded FFT size; called by ParSetup (comm.c:489-491) */
int fftFit(int x, int divis);
/* CheckNprocs, src/fft.c:489: the GPU build runs one process per GPU */
void CheckNprocs(void);
/* InitDmatrix, src/fft.c:918: builds the device context and D on the GPU; honours prognosis */
void InitDmatrix(void);
/* Free_FFT_Dmat, src/fft.c:1420 */
void Free_FFT_Dmat(void);
/* MatVec, src/matvec.c:128: host vectors of local_nRows complex; argvec unchanged; inprod = |resultvec|^2 */
void MatVec(doublecomplex *argvec, doublecomplex *resultvec, double *inprod, bool her, clock_t *timing,
	clock_t *comm_timing);
/* IterativeSolver, src/iterative.c:1398: solves for Einc (host), leaves xvec and pvec (host), prints RE_ lines */
int IterativeSolver(enum iter method, enum incpol which);
/* CalcField, src/crosssec.c:801, reached through the linker's --wrap=CalcField (so the reference's crosssec.c stays
 * unchanged): the scattering amplitude in direction n from the polarisations of the last IterativeSolver, on the GPU
 * (CalcFieldFree, crosssec.c:506-596) for free space with the Draine/FINDIP relations; surface mode and the
 * second-order relations go to the reference's own routine (__real_CalcField). */
void __wrap_CalcField(doublecomplex ebuff[3], const double n[3]);

#endif
