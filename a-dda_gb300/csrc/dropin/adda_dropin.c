/* adda_dropin.c - the reference's fft.c / matvec.c / iterative.c entry points, implemented on libadda_gb300.
 *
 * Link this object and libadda_gb300.so instead of the reference's fft.c, matvec.c and iterative.c (all other
 * reference sources unchanged): the host parses the command line, builds the particle and the incident beam, and
 * calls InitDmatrix / IterativeSolver / Free_FFT_Dmat exactly as before (calculator.c:685,563; CalculateE.c:860);
 * the D matrix, every matvec and the whole Krylov solve then run on the GPU, and xvec/pvec come back to the host for
 * the reference's own cross sections and scattering output.
 *
 * The reference's globals, types and host services used here are declared below with the file that defines them; they
 * must match the reference's sequential build (FFTW3 branch, no MPI).
 *
 * Environment (the reference's command line is left unchanged):
 *   ADDA_GB300_PREC=fp64|mixed   arithmetic of IterativeSolver (default fp64, the reference's)
 *   ADDA_GB300_DEVICE=<n>        CUDA device (default 0)
 * Supported: -int poi|fcd|fcd_st|nloc|nloc_av|igt_so|so (with every -pol the host computes), -surf with -int_surf img|som
 * (the reflected tensor comes from the host's ReflTerm_int), every -iter method, -init_field auto|zero|inc|read|wkb,
 * -chpoint/-chp_load (FP64), and the scattered fields of CalcField, CalcAlldir and CalcScatGrid (free space).
 * Refused with the reference's LogError: -int igt, -no_reduced_fft, more than one MPI process.
 */
#include "adda_gb300.h"
#include "adda_dropin.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAX_NMAT 15 /* const.h:106 */
enum enwho { ALL, ONE };                                           /* const.h:406-409 */
enum ec { EC_OK, EC_ERROR, EC_WARN, EC_INFO };                     /* const.h:418-423 */
enum inter { G_FCD, G_FCD_ST, G_IGT, G_IGT_SO, G_NLOC, G_NLOC_AV, G_POINT_DIP, G_SO }; /* const.h:212-224 */
enum init_field { IF_AUTO, IF_ZERO, IF_INC, IF_READ, IF_WKB };     /* const.h:321-327 */
enum chpoint { CHP_NONE, CHP_NORMAL, CHP_REGULAR, CHP_ALWAYS };     /* const.h:313-319 */
#define CHP_EXIT -2                                                  /* const.h:330 */
#define UNDEF -1                                                     /* const.h:47 */

/* globals of the reference host: vars.c, param.c, timing.c, calculator.c */
extern int boxX, boxY, boxZ, nprocs, Nmat, maxiter;
extern size_t gridX, gridY, gridZ, gridYZ, local_Nsmall, local_nvoid_Ndip, local_nRows;
extern double gridspace, WaveNum, memory;
extern bool prognosis, reduced_FFT, surface, orient_avg, ipr_required;
extern enum inter IntRelation;
extern bool msubInf;                                                  /* vars.c:128 */
extern doublecomplex msub;                                            /* vars.c:126 */
extern double ZsumShift;                                              /* make_particle.c:68 */
/* the reflected Green's tensor of the -int_surf relation chosen by InitInteraction (interaction.h:39) */
extern void (*ReflTerm_int)(const int i, const int j, const int k, doublecomplex result[static restrict 6]);
extern const double nloc_Rp; /* param.c:132 */
extern FILE *logfile;
extern unsigned short *position;
extern unsigned char *material;
extern doublecomplex cc_sqrt[MAX_NMAT][3];
extern doublecomplex *xvec, *pvec, *Einc;
extern doublecomplex ref_index[MAX_NMAT], chi_inv[MAX_NMAT][3];
extern double prop[3];
extern const char *infi_fnameY, *infi_fnameX;
void ReadField(const char *fname, doublecomplex *field); /* comm.c:562 */
extern const double iter_eps;
extern const enum init_field InitField;
extern const bool recalc_resid;
extern const enum chpoint chp_type;                                  /* param.c:142-144 */
extern const time_t chp_time;
extern const char *chp_dir;
extern bool load_chpoint;                                            /* vars.c:54 */
extern const char *directory;                                        /* vars.c:71 */
extern int ringid;                                                   /* vars.c:100 */
extern time_t last_chp_wt;                                           /* timing.c:60 */
extern clock_t Timing_Dm_Init, Timing_FFT_Init, Timing_OneIter, Timing_InitIter, Timing_MVP;
extern size_t TotalIter, TotalMatVec;
/* host services: io.c */
void LogError(enum enwho who, const char *srcfile, int srcline, const char *fmt, ...);
void LogWarning(enum ec code, enum enwho who, const char *srcfile, int srcline, const char *fmt, ...);
void PrintBoth(FILE *file, const char *fmt, ...);
void MkDirErr(const char *dir, enum enwho who, const char *srcfile, int srcline);

/* the reference's fft.c also defines these globals; other reference files may name them */
doublecomplex *Xmatrix, *Dmatrix, *slices, *slices_tr;
double *BT_buffer, *BT_rbuffer;

#define ERR(...) LogError(ONE, __FILE__, __LINE__, __VA_ARGS__)

static adda_gb300_ctx *g_ctx;
static int g_method; /* ADDA_ITER_* of the current IterativeSolver */
/* the device polarisations belong to the host's pvec of the last IterativeSolver */
static int g_pvec_valid = 0;
static doublecomplex g_ccs[MAX_NMAT][3];
static int g_ccs_valid;

static int env_prec(void)
{
	const char *p = getenv("ADDA_GB300_PREC");
	return (p && !strcmp(p, "mixed")) ? ADDA_PREC_MIXED : ADDA_PREC_FP64;
}

int fftFit(int x, int divis)
{
	return adda_gb300_fft_fit(x, divis);
}

void CheckNprocs(void)
{
	if (nprocs != 1) ERR("The GPU build runs one process per GPU; %d processes were started", nprocs);
}

void InitDmatrix(void)
{
	clock_t start = clock();
	int inter = ADDA_INT_POI;
	if (IntRelation == G_POINT_DIP) inter = ADDA_INT_POI;
	else if (IntRelation == G_FCD) inter = ADDA_INT_FCD;
	else if (IntRelation == G_FCD_ST) inter = ADDA_INT_FCD_ST;
	else if (IntRelation == G_NLOC) inter = ADDA_INT_NLOC;
	else if (IntRelation == G_NLOC_AV) inter = ADDA_INT_NLOC_AV;
	else if (IntRelation == G_IGT_SO) inter = ADDA_INT_IGT_SO;
	else if (IntRelation == G_SO) inter = ADDA_INT_SO;
	else ERR("The GPU build supports the interaction terms -int poi|fcd|fcd_st|nloc|nloc_av|igt_so|so only");
	/* -int so turns the reduced FFT off in the reference (param.c:1992-1996) for its general, non-averaged form; the
	 * averaged form it uses has the point-dipole reflection symmetries, so the GPU keeps the reduced D for it */
	if (!reduced_FFT && inter != ADDA_INT_SO) ERR("The GPU build requires the reduced FFT (do not use -no_reduced_fft)");
	local_Nsmall = (gridX / 2) * (gridYZ / 2); /* fft.c:975 with nprocs=1 */
	if (logfile) fprintf(logfile, "The FFT grid is: %zux%zux%zu\n", gridX, gridY, gridZ);
	/* device memory of the matvec (D in FP64+FP32, expanded grid, chunk buffer) for the log */
	double dlen = 6.0 * gridX * (gridY / 2 + 1) * (gridZ / 2 + 1);
	double mem = 24 * dlen + 16.0 * 3 * gridX * boxY * boxZ;
	PrintBoth(logfile, "Memory usage for MatVec matrices (GPU): %.1f MB\n", mem / (1024.0 * 1024.0));
	if (prognosis) return;
	adda_gb300_problem p;
	memset(&p, 0, sizeof(p));
	p.boxX = boxX; p.boxY = boxY; p.boxZ = boxZ;
	p.gridX = (int)gridX; p.gridY = (int)gridY; p.gridZ = (int)gridZ;
	p.ndip = local_nvoid_Ndip;
	p.position = position;
	p.material = material;
	p.gridspace = gridspace;
	p.wavenum = WaveNum;
	p.nrhs_max = 1;
	p.device = getenv("ADDA_GB300_DEVICE") ? atoi(getenv("ADDA_GB300_DEVICE")) : 0;
	p.interaction = inter;
	static double tables[ADDA_GB300_INT_TABLES];
	if (inter == ADDA_INT_IGT_SO || inter == ADDA_INT_SO) { /* the reference reads tables/t*f.dat (const.h:274) */
		if (adda_gb300_read_int_tables("tables", tables)) ERR("cannot read the integral tables tables/t1f.dat..t10f.dat");
		p.int_tables = tables;
		p.so_m_re = creal(ref_index[0]);
		p.so_m_im = cimag(ref_index[0]);
	}
	p.nloc_rp = nloc_Rp;
	doublecomplex *gr = NULL;
	if (surface) {
		/* the reflected tensor of every in-plane offset and height sum, from the reference's own ReflTerm_int (image
		 * dipole or Sommerfeld integrals, as InitRmatrix evaluates it, fft.c:846-850); the GPU transforms it */
		const size_t nk = 2 * (size_t)boxZ - 1, ni = 2 * (size_t)boxX - 1;
		gr = malloc(sizeof(doublecomplex) * 6 * nk * boxY * ni);
		if (!gr) ERR("cannot allocate the reflected Green's tensor (%zu MB)", 96 * nk * boxY * ni >> 20);
		for (int k = 0; k < (int)nk; k++)
			for (int j = 0; j < boxY; j++)
				for (int i = 1 - boxX; i < boxX; i++)
					(*ReflTerm_int)(i, j, k, gr + 6 * (((size_t)k * boxY + j) * ni + (size_t)(i + boxX - 1)));
		p.surface = 1;
		p.zsum_shift = ZsumShift;
		p.msub_re = creal(msub);
		p.msub_im = cimag(msub);
		p.msub_inf = msubInf;
		p.refl = ADDA_REFL_HOST;
		p.refl_data = (const double *)gr;
	}
	const int crc = adda_gb300_create(&p, &g_ctx);
	free(gr);
	if (crc) ERR("GPU initialisation failed: %s", adda_gb300_last_error());
	if (adda_gb300_init_dmatrix(g_ctx)) ERR("GPU D-matrix initialisation failed: %s", adda_gb300_last_error());
	g_ccs_valid = 0;
	g_pvec_valid = 0;
	Timing_Dm_Init = clock() - start;
	Timing_FFT_Init = 0;
}

void Free_FFT_Dmat(void)
{
	if (g_ctx) adda_gb300_destroy(g_ctx);
	g_ctx = NULL;
	g_pvec_valid = 0;
}

/* InitCC (calculator.c:266) may change cc_sqrt between the two polarisations: upload when it changed */
static void sync_cc(void)
{
	if (g_ccs_valid && !memcmp(g_ccs, cc_sqrt, sizeof(g_ccs))) return;
	if (adda_gb300_set_cc_sqrt(g_ctx, 0, Nmat, (const double *)cc_sqrt))
		ERR("GPU: %s", adda_gb300_last_error());
	memcpy(g_ccs, cc_sqrt, sizeof(g_ccs));
	g_ccs_valid = 1;
}

void MatVec(doublecomplex *argvec, doublecomplex *resultvec, double *inprod, bool her, clock_t *timing,
	clock_t *comm_timing)
{
	(void)comm_timing;
	clock_t t0 = clock();
	if (inprod && !ipr_required) ERR("Incompatibility error in MatVec"); /* matvec.c:184 */
	if (!g_ctx) ERR("MatVec called before InitDmatrix");
	sync_cc();
	if (adda_gb300_matvec(g_ctx, ADDA_PREC_FP64, 1, (const double *)argvec, (double *)resultvec, inprod, her))
		ERR("GPU MatVec failed: %s", adda_gb300_last_error());
	*timing += clock() - t0;
	TotalMatVec++;
}

/* ProgressReport output format, iterative.c:69-70, 295-305 */
static void report(int niter, double err, double prev_err, int counter)
{
	double progr = 1 - err / prev_err;
	const char *tag = (counter == 0) ? "+ " : (progr > 0 ? "-+" : "- ");
	if (!orient_avg && logfile) fprintf(logfile, "RE_%03d = %.10E  %s  progress =% .6f\n", niter, err, tag, progr);
	printf("RE_%03d = %.10E  %s\n", niter, err, tag);
}

/* SaveIterChpoint (iterative.c:165-218): <chp_dir>/chp.log and <chp_dir>/chp.<ringid> in the reference's format */
static void save_chpoint(void)
{
	char fname[4096];
	snprintf(fname, sizeof(fname), "%s/chp.log", chp_dir);
	FILE *f = fopen(fname, "w");
	if (!f) {
		MkDirErr(chp_dir, ONE, __FILE__, __LINE__);
		f = fopen(fname, "w");
	}
	if (!f) ERR("Failed to open file '%s'", fname);
	fprintf(f, "Info about the run, which produced the checkpoint, can be found in ../%s", directory);
	fclose(f);
	size_t n = adda_gb300_chpoint_size(g_ctx, g_method);
	unsigned char *buf = malloc(n);
	if (!buf || adda_gb300_chpoint_save(g_ctx, 0, buf, n)) ERR("GPU checkpoint failed: %s", adda_gb300_last_error());
	snprintf(fname, sizeof(fname), "%s/chp.%d", chp_dir, ringid);
	if (!(f = fopen(fname, "wb"))) ERR("Failed to open file '%s'", fname);
	if (fwrite(buf, 1, n, f) != n) ERR("Failed writing to file '%s'", fname);
	fclose(f);
	free(buf);
	PrintBoth(logfile, "Checkpoint (iteration) saved\n");
}

/* LoadIterChpoint (iterative.c:222-278): the file is checked by the library and applied by the next solve */
static void load_chpoint_file(void)
{
	char fname[4096];
	snprintf(fname, sizeof(fname), "%s/chp.%d", chp_dir, ringid);
	FILE *f = fopen(fname, "rb");
	if (!f) ERR("Failed to open file '%s'", fname);
	fseek(f, 0, SEEK_END);
	const long n = ftell(f);
	fseek(f, 0, SEEK_SET);
	unsigned char *buf = malloc(n > 0 ? (size_t)n : 1);
	if (n <= 0 || fread(buf, 1, (size_t)n, f) != (size_t)n) ERR("Failed reading from file '%s'", fname);
	fclose(f);
	int ind;
	memcpy(&ind, buf, sizeof(int));
	const int ind_of[7] = {5, 2, 1, 3, 4, 6, 0}; /* params table order, iterative.c:118-125 */
	if (ind != ind_of[g_method]) ERR("File '%s' is for different iterative method", fname);
	if (adda_gb300_chpoint_load(g_ctx, 0, buf, (size_t)n)) ERR("File '%s': %s", fname, adda_gb300_last_error());
	free(buf);
	PrintBoth(logfile, "Checkpoint (iteration) loaded\n");
}

int IterativeSolver(enum iter method, enum incpol which)
{
	adda_gb300_solve_params sp;
	memset(&sp, 0, sizeof(sp));
	if (method == IT_QMR_CS) sp.method = ADDA_ITER_QMR_CS;
	else if (method == IT_BICGSTAB) sp.method = ADDA_ITER_BICGSTAB;
	else if (method == IT_BICG_CS) sp.method = ADDA_ITER_BICG_CS;
	else if (method == IT_CGNR) sp.method = ADDA_ITER_CGNR;
	else if (method == IT_CSYM) sp.method = ADDA_ITER_CSYM;
	else if (method == IT_QMR_CS_2) sp.method = ADDA_ITER_QMR_CS_2;
	else if (method == IT_BCGS2) sp.method = ADDA_ITER_BCGS2;
	else ERR("Unknown -iter method for the GPU build");
	if (InitField == IF_AUTO) sp.init_field = ADDA_IF_AUTO;
	else if (InitField == IF_ZERO) sp.init_field = ADDA_IF_ZERO;
	else if (InitField == IF_INC) sp.init_field = ADDA_IF_INC;
	else if (InitField == IF_READ || InitField == IF_WKB) {
		/* CalcInitField (iterative.c:1380-1392): a field E in xvec -- read from file (ReadField, comm.c:562) or
		 * the WKB approximation -- turned into x_0 = E/(cc_sqrt*chi_inv) (InitFieldfromE, iterative.c:1325-1332) */
		if (InitField == IF_READ) ReadField(which == INCPOL_Y ? infi_fnameY : infi_fnameX, xvec);
		else {
			if (prop[2] != 1)
				ERR("WKB initial field currently works only with default incident direction of the incoming wave "
					"(along z-axis)");
			double ri[2 * MAX_NMAT];
			for (int i = 0; i < Nmat; i++) {
				ri[2 * i] = creal(ref_index[i]);
				ri[2 * i + 1] = cimag(ref_index[i]);
			}
			if (adda_gb300_wkb_field(boxX, boxY, boxZ, local_nvoid_Ndip, position, material, Nmat, ri,
					WaveNum * gridspace, (const double *)Einc, (double *)xvec))
				ERR("WKB initial field failed: %s", adda_gb300_last_error());
		}
		for (size_t i = 0; i < local_nvoid_Ndip; i++)
			for (int a = 0; a < 3; a++)
				xvec[3 * i + a] /= cc_sqrt[material[i]][a] * chi_inv[material[i]][a];
		sp.init_field = ADDA_IF_X0;
	}
	else ERR("Unknown -init_field for the GPU build");
	if (!g_ctx) ERR("IterativeSolver called before InitDmatrix");
	sp.precision = env_prec();
	sp.eps = iter_eps;
	sp.maxiter = maxiter;
	g_method = sp.method;
	/* checkpoints (iterative.c:165-278,308-317,1498) work on the FP64 solver state */
	if ((load_chpoint || chp_type != CHP_NONE) && sp.precision != ADDA_PREC_FP64)
		ERR("Checkpoints need ADDA_GB300_PREC=fp64 in the GPU build");
	if (load_chpoint) {
		load_chpoint_file();
		sp.init_field = ADDA_IF_CHPOINT;
	}
	if (chp_type == CHP_ALWAYS) sp.full_steps = 1; /* no half-step exit of BiCGStab (iterative.c:703) */
	clock_t t0 = clock();
	sync_cc();
	const int cap = (maxiter < 100000 ? maxiter : 100000) + 2;
	double *hist = calloc((size_t)cap, sizeof(double));
	adda_gb300_rhs_stats st;
	int chp_exit = 0, first = 1, matvecs = 0;
	for (;;) {
		/* -chpoint <time>: the time left until the next checkpoint, counted from the last one (timing.c:102) */
		if (chp_type != CHP_NONE && chp_time != UNDEF) {
			const double left = (double)chp_time - difftime(time(NULL), last_chp_wt);
			sp.chp_time = left > 0 ? left : 1e-9;
		}
		int rc = adda_gb300_solve(g_ctx, &sp, 1, (const double *)Einc, (double *)xvec, (double *)pvec, &st, hist,
			cap);
		if (rc < 0) ERR("GPU IterativeSolver failed: %s", adda_gb300_last_error());
		matvecs += st.matvecs_fp64 + st.matvecs_fp32;
		/* print the initial field choice and the residual history like IterativeSolver/ProgressReport */
		if (sp.precision == ADDA_PREC_FP64) {
			int i0 = 1;
			if (sp.init_field == ADDA_IF_CHPOINT) {
				/* resumed: the history continues after the saved iteration (hist[k] = RE_k) */
				while (i0 < cap && hist[i0 - 1] == 0) i0++;
				first = 0;
			}
			if (first) {
				const char *descr = (sp.init_field == ADDA_IF_ZERO ||
					(sp.init_field == ADDA_IF_AUTO && hist[0] == 1.0)) ? "x_0 = 0\n" : "x_0 = E_inc\n";
				char fdescr[512];
				if (InitField == IF_WKB) descr = "x_0 = result of WKB\n"; /* iterative.c:1383,1390 */
				else if (InitField == IF_READ) {
					snprintf(fdescr, sizeof(fdescr), "x_0 = from file %s\n",
						which == INCPOL_Y ? infi_fnameY : infi_fnameX);
					descr = fdescr;
				}
				if (!orient_avg && logfile) fprintf(logfile, "%sRE_%03d = %.10E\n", descr, 0, hist[0]);
				printf("%sRE_%03d = %.10E\n", descr, 0, hist[0]);
			}
			double best = hist[i0 - 1], prev = hist[i0 - 1];
			int counter = 0;
			for (int i = i0; i <= st.niter && i < cap; i++) {
				if (hist[i] <= best) { best = hist[i]; counter = 0; }
				else counter++;
				report(i, hist[i], prev, counter);
				prev = hist[i];
			}
		}
		else {
			PrintBoth(logfile, "Mixed precision: %d FP32 iterations, %d FP64 refinement steps, final FP64 residual "
				"RE = %.10E\n", st.niter, st.refinements, st.resid);
		}
		if (st.status != ADDA_GB300_CHPOINT) break;
		/* the checkpoint time has passed (ProgressReport, iterative.c:308-317) */
		save_chpoint();
		time(&last_chp_wt);
		if (chp_type != CHP_REGULAR) {
			chp_exit = 1;
			break;
		}
		/* regular checkpoints: carry on from the state just saved */
		size_t n = adda_gb300_chpoint_size(g_ctx, g_method);
		unsigned char *buf = malloc(n);
		if (!buf || adda_gb300_chpoint_save(g_ctx, 0, buf, n) || adda_gb300_chpoint_load(g_ctx, 0, buf, n))
			ERR("GPU checkpoint failed: %s", adda_gb300_last_error());
		free(buf);
		sp.init_field = ADDA_IF_CHPOINT;
		first = 0;
	}
	if (chp_type == CHP_ALWAYS && !chp_exit) save_chpoint(); /* iterative.c:1498 */
	free(hist);
	if (st.status == ADDA_GB300_EBREAKDOWN) ERR("Krylov solver breakdown on the GPU (iteration %d)", st.niter);
	if (st.status == ADDA_GB300_ESTAGNATION)
		ERR("Residual norm haven't decreased for maximum allowed number of iterations");
	if (st.status == ADDA_GB300_EMAXITER)
		LogWarning(EC_WARN, ONE, __FILE__, __LINE__, "Iterations haven't converged in %d iterations. Further "
			"calculated scattering quantities may be less accurate.", maxiter);
	if (recalc_resid) { /* iterative.c:1512-1520: |A.x - b|^2 / |b|^2 with the FP64 matvec */
		doublecomplex *ax = malloc(sizeof(doublecomplex) * local_nRows);
		clock_t tm = 0;
		MatVec(xvec, ax, NULL, false, &tm, NULL);
		double num = 0, den = 0;
		for (size_t i = 0; i < local_nvoid_Ndip; i++)
			for (int c = 0; c < 3; c++) {
				doublecomplex b = cc_sqrt[material[i]][c] * Einc[3 * i + c];
				doublecomplex d = ax[3 * i + c] - b;
				num += creal(d) * creal(d) + cimag(d) * cimag(d);
				den += creal(b) * creal(b) + cimag(b) * cimag(b);
			}
		free(ax);
		if (!orient_avg && logfile) fprintf(logfile, "Final (recalculated) residual norm: %.10E\n", sqrt(num / den));
		printf("Final (recalculated) residual norm: %.10E\n", sqrt(num / den));
	}
	TotalIter += (size_t)st.niter;
	TotalMatVec += (size_t)matvecs;
	Timing_InitIter = 0;
	Timing_MVP = clock() - t0;
	Timing_OneIter = st.niter ? (clock() - t0) / st.niter : 0;
	g_pvec_valid = 1;
	if (chp_exit) return CHP_EXIT; /* iterative.c:1528 */
	return st.niter;
}

extern const enum scat ScatRelation;
void __real_CalcField(doublecomplex ebuff[3], const double n[3]);

void __wrap_CalcField(doublecomplex ebuff[3], const double n[3])
{
	if (g_ctx && g_pvec_valid && !surface && (ScatRelation == SQ_DRAINE || ScatRelation == SQ_FINDIP)) {
		if (adda_gb300_scattered_fields(g_ctx, 1, 1, n, (double *)ebuff))
			ERR("GPU CalcField failed: %s", adda_gb300_last_error());
		return;
	}
	__real_CalcField(ebuff, n);
}

/* CalcAlldir (crosssec.c:991-1050): the scattered field on the whole alldir grid, here in one batch on the GPU; the
 * directions and the Epar/Eper unit vectors come from the reference's own SetScatPlane (crosssec.c:944-990), the
 * host's Romberg integration (ScaCross, AsymParm_x/y/z) then reads E2_alldir as usual */
typedef struct {
	double min, max;
	size_t N;
	double *val;
} angle_set; /* types.h:44-50 */
extern angle_set theta_int, phi_int;           /* crosssec.c:62 */
extern doublecomplex *E_ad;                    /* calculator.c:68-69 */
extern double *E2_alldir;
void SetScatPlane(const double ct, const double st, const double phi, double robs[3], double polPer[3]);
void __real_CalcAlldir(void);

void __wrap_CalcAlldir(void)
{
	if (!(g_ctx && g_pvec_valid && !surface && (ScatRelation == SQ_DRAINE || ScatRelation == SQ_FINDIP))) {
		__real_CalcAlldir();
		return;
	}
	const double deg = 0.017453292519943295769236907684886; /* Deg2Rad */
	const size_t np = theta_int.N * phi_int.N;
	double *dirs = malloc(sizeof(double) * 9 * np), *per = dirs + 3 * np, *par = dirs + 6 * np;
	doublecomplex *e = malloc(sizeof(doublecomplex) * 3 * np);
	if (!dirs || !e) ERR("CalcAlldir: out of host memory");
	printf("Calculating scattered field for the whole solid angle:\n");
	for (size_t i = 0, q = 0; i < theta_int.N; i++) {
		const double th = deg * theta_int.val[i], ct = cos(th), st = sin(th);
		for (size_t j = 0; j < phi_int.N; j++, q++) {
			double *r = dirs + 3 * q, *u = per + 3 * q, *w = par + 3 * q;
			SetScatPlane(ct, st, deg * phi_int.val[j], r, u);
			w[0] = r[1] * u[2] - r[2] * u[1]; /* Epar = robserver x Eper */
			w[1] = r[2] * u[0] - r[0] * u[2];
			w[2] = r[0] * u[1] - r[1] * u[0];
		}
	}
	if (adda_gb300_scattered_fields(g_ctx, 1, (int)np, dirs, (double *)e))
		ERR("GPU CalcAlldir failed: %s", adda_gb300_last_error());
	for (size_t q = 0; q < np; q++) {
		doublecomplex a = 0, b = 0;
		for (int k = 0; k < 3; k++) {
			a += e[3 * q + k] * per[3 * q + k];
			b += e[3 * q + k] * par[3 * q + k];
		}
		E_ad[2 * q] = a;
		E_ad[2 * q + 1] = b;
		E2_alldir[q] = creal(a) * creal(a) + cimag(a) * cimag(a) + creal(b) * creal(b) + cimag(b) * cimag(b);
	}
	printf("  done\n");
	free(dirs);
	free(e);
}

/* CalcScatGrid (crosssec.c:1055-1100): the field on the -scat_grid_inp grid (a theta x phi grid or theta/phi pairs)
 * in one GPU batch, projected on Eper/Epar from the reference's SetScatPlane, into EgridY or EgridX */
enum scatgrid { SG_GRID, SG_PAIRS };           /* const.h:291-294 */
typedef struct {
	enum scatgrid type;
	size_t N;
	angle_set theta, phi;
} scat_grid_angles;                            /* types.h:52-58 */
extern scat_grid_angles angles;                /* vars.c:95-97 */
extern doublecomplex *EgridX, *EgridY;
void __real_CalcScatGrid(enum incpol which);

void __wrap_CalcScatGrid(enum incpol which)
{
	if (!(g_ctx && g_pvec_valid && !surface && (ScatRelation == SQ_DRAINE || ScatRelation == SQ_FINDIP))) {
		__real_CalcScatGrid(which);
		return;
	}
	const double deg = 0.017453292519943295769236907684886;
	const size_t np = angles.N, nph = (angles.type == SG_GRID) ? angles.phi.N : 1;
	double *dirs = malloc(sizeof(double) * 9 * np), *per = dirs + 3 * np, *par = dirs + 6 * np;
	doublecomplex *e = malloc(sizeof(doublecomplex) * 3 * np);
	if (!dirs || !e) ERR("CalcScatGrid: out of host memory");
	printf("Calculating grid of scattered field:\n");
	size_t q = 0;
	for (size_t i = 0; i < angles.theta.N && q < np; i++) {
		const double th = deg * angles.theta.val[i], ct = cos(th), st = sin(th);
		for (size_t j = 0; j < nph && q < np; j++, q++) {
			const double ph = deg * ((angles.type == SG_GRID) ? angles.phi.val[j] : angles.phi.val[i]);
			double *r = dirs + 3 * q, *u = per + 3 * q, *w = par + 3 * q;
			SetScatPlane(ct, st, ph, r, u);
			w[0] = r[1] * u[2] - r[2] * u[1];
			w[1] = r[2] * u[0] - r[0] * u[2];
			w[2] = r[0] * u[1] - r[1] * u[0];
		}
	}
	if (adda_gb300_scattered_fields(g_ctx, 1, (int)q, dirs, (double *)e))
		ERR("GPU CalcScatGrid failed: %s", adda_gb300_last_error());
	doublecomplex *grid = (which == INCPOL_Y) ? EgridY : EgridX;
	for (size_t k = 0; k < q; k++) {
		doublecomplex a = 0, b = 0;
		for (int c = 0; c < 3; c++) {
			a += e[3 * k + c] * per[3 * k + c];
			b += e[3 * k + c] * par[3 * k + c];
		}
		grid[2 * k] = a;
		grid[2 * k + 1] = b;
	}
	printf("  done\n");
	free(dirs);
	free(e);
}
