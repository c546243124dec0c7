/* mock_host.c - a minimal stand-in for the reference's C host, for testing the drop-in layer (adda_dropin.c) where
 * the reference sources are not available. It defines the reference globals the drop-in reads (with the reference's
 * names and types, vars.c / param.c / timing.c / calculator.c), the three io.c services it calls, and a main() that
 * drives the drop-in exactly like Calculator/CalculateE do: ParSetup's fftFit, InitDmatrix, IterativeSolver,
 * MatVec, Free_FFT_Dmat. Inputs come from libadda_gb300's host-side setup.
 *
 * usage: mock_host <grid> <m_re> <m_im> <dpl> <method> <eps_exponent> <out.bin> [wkb | read <field.bin> |
 *        chpoint <dir> <normal|regular|always> <seconds> [maxiter] | chp_load <dir>]
 * writes: ndip (int64), then pvec and a MatVec of Einc (complex doubles, 3*ndip each)
 * read: the field file holds 3*ndip complex doubles (the mock's ReadField; the reference's reads io.c's text format)
 */
#include "adda_gb300.h"
#include "adda_dropin.h"

#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <sys/stat.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum enwho { ALL, ONE };
enum ec { EC_OK, EC_ERROR, EC_WARN, EC_INFO };
enum inter { G_FCD, G_FCD_ST, G_IGT, G_IGT_SO, G_NLOC, G_NLOC_AV, G_POINT_DIP, G_SO };
enum init_field { IF_AUTO, IF_ZERO, IF_INC, IF_READ, IF_WKB };
enum chpoint { CHP_NONE, CHP_NORMAL, CHP_REGULAR, CHP_ALWAYS };

int boxX, boxY, boxZ, nprocs = 1, Nmat = 1, maxiter = 100000;
size_t gridX, gridY, gridZ, gridYZ, local_Nsmall, local_nvoid_Ndip, local_nRows;
double gridspace, WaveNum, memory;
bool prognosis = false, reduced_FFT = true, surface = false, orient_avg = false, ipr_required = false;
enum inter IntRelation = G_POINT_DIP;
/* surface mode: the substrate and the image-dipole relation (ReflTerm_img, interaction.c:1092-1153), stand-ins for
 * vars.c:126-129, make_particle.c:68 and InitInteraction */
bool msubInf = false;
doublecomplex msub;
double ZsumShift, hsub;
static doublecomplex surfRCn;
static void refl_img(const int i, const int j, const int k, doublecomplex g[static restrict 6])
{
	const double q[3] = {i, j, k + ZsumShift};
	double rr = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
	const double v[3] = {q[0] / rr, q[1] / rr, q[2] / rr};
	const double qm[6] = {v[0] * v[0], v[0] * v[1], v[0] * v[2], v[1] * v[1], v[1] * v[2], v[2] * v[2]};
	rr *= gridspace;
	const double kr = WaveNum * rr, kr2 = kr * kr, t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
	const doublecomplex scale = surfRCn * cexp(I * kr) / (rr * rr * rr);
	for (int a = 0; a < 6; a++)
		g[a] = (a == 0 || a == 3 || a == 5) ? ((t1 * qm[a] + t3) + I * (kr + t2 * qm[a])) * scale
			: (t1 + I * t2) * qm[a] * scale;
	g[2] = -g[2];
	g[4] = -g[4];
	g[5] = -g[5];
}
void (*ReflTerm_int)(const int i, const int j, const int k, doublecomplex result[static restrict 6]) = refl_img;
double nloc_Rp = 0;
FILE *logfile;
unsigned short *position;
unsigned char *material;
doublecomplex cc_sqrt[15][3];
doublecomplex *xvec, *pvec, *Einc;
double iter_eps = 1e-5;
enum init_field InitField = IF_AUTO;
doublecomplex ref_index[15], chi_inv[15][3];
double prop[3], incPolX[3], incPolY[3];
typedef struct {
	double min, max;
	size_t N;
	double *val;
} angle_set;
angle_set theta_int, phi_int;
doublecomplex *E_ad;
double *E2_alldir;
void CalcAlldir(void);
enum scatgrid { SG_GRID, SG_PAIRS };
typedef struct {
	enum scatgrid type;
	size_t N;
	angle_set theta, phi;
} scat_grid_angles;
scat_grid_angles angles;
doublecomplex *EgridX, *EgridY;
void CalcScatGrid(enum incpol which);
const char *infi_fnameY, *infi_fnameX;
enum chpoint chp_type = CHP_NONE;
time_t chp_time = -1, last_chp_wt;
const char *chp_dir = "chpoint", *directory = "run000";
bool load_chpoint = false;
int ringid = 0;

void MkDirErr(const char *dir, enum enwho who, const char *srcfile, int srcline)
{
	(void)who; (void)srcfile; (void)srcline;
	if (mkdir(dir, 0755) == -1 && errno != EEXIST) {
		fprintf(stderr, "ERROR: Failed to make directory '%s'\n", dir);
		exit(1);
	}
}

void ReadField(const char *fname, doublecomplex *field)
{
	FILE *f = fopen(fname, "rb");
	if (!f || fread(field, sizeof(doublecomplex), local_nRows, f) != local_nRows) {
		fprintf(stderr, "ERROR: cannot read %s\n", fname);
		exit(1);
	}
	fclose(f);
}
enum scat ScatRelation = SQ_DRAINE;
/* the reference's CalcField lives in another object (mock_crosssec.c, like crosssec.c), so that this file's calls
 * go through the linker's --wrap=CalcField */
void CalcField(doublecomplex ebuff[3], const double n[3]);
bool recalc_resid = true;
clock_t Timing_Dm_Init, Timing_FFT_Init, Timing_OneIter, Timing_InitIter, Timing_MVP;
size_t TotalIter, TotalMatVec;

void LogError(enum enwho who, const char *srcfile, int srcline, const char *fmt, ...)
{
	(void)who;
	va_list a;
	va_start(a, fmt);
	fprintf(stderr, "ERROR: (%s:%d) ", srcfile, srcline);
	vfprintf(stderr, fmt, a);
	fprintf(stderr, "\n");
	va_end(a);
	exit(1);
}

void LogWarning(enum ec code, enum enwho who, const char *srcfile, int srcline, const char *fmt, ...)
{
	(void)code; (void)who; (void)srcfile; (void)srcline;
	va_list a;
	va_start(a, fmt);
	fprintf(stderr, "WARNING: ");
	vfprintf(stderr, fmt, a);
	fprintf(stderr, "\n");
	va_end(a);
}

void PrintBoth(FILE *file, const char *fmt, ...)
{
	va_list a;
	va_start(a, fmt);
	if (file) vfprintf(file, fmt, a);
	va_end(a);
	va_start(a, fmt);
	vprintf(fmt, a);
	va_end(a);
}

int main(int argc, char **argv)
{
	if (argc < 8) return 2;
	const int grid = atoi(argv[1]);
	const double mre = atof(argv[2]), mim = atof(argv[3]), dpl = atof(argv[4]);
	/* -iter names of param.c:1232-1238 */
	const char *names[] = {"bcgs2", "bicg", "bicgstab", "cgnr", "csym", "qmr", "qmr2"};
	const enum iter ids[] = {IT_BCGS2, IT_BICG_CS, IT_BICGSTAB, IT_CGNR, IT_CSYM, IT_QMR_CS, IT_QMR_CS_2};
	enum iter method = IT_QMR_CS;
	for (int i = 0; i < 7; i++)
		if (!strcmp(argv[5], names[i])) method = ids[i];
	iter_eps = pow(10, -atof(argv[6]));
	logfile = stdout;
	CheckNprocs();
	if (adda_gb300_fit_box(ADDA_SHAPE_SPHERE, NULL, grid, &boxY, &boxZ)) return 3;
	boxX = grid;
	local_nvoid_Ndip = adda_gb300_make_particle(ADDA_SHAPE_SPHERE, NULL, boxX, boxY, boxZ, NULL, NULL);
	local_nRows = 3 * local_nvoid_Ndip;
	position = malloc(sizeof(unsigned short) * local_nRows);
	material = malloc(local_nvoid_Ndip);
	adda_gb300_make_particle(ADDA_SHAPE_SPHERE, NULL, boxX, boxY, boxZ, position, material);
	gridX = fftFit(2 * boxX, 1); /* ParSetup, comm.c:489-491 */
	gridY = fftFit(2 * boxY, 1);
	gridZ = fftFit(2 * boxZ, 2);
	gridYZ = gridY * gridZ;
	WaveNum = 1.0;
	gridspace = 2 * M_PI / dpl;
	double *py = incPolY, *px = incPolX, cc[6];
	adda_gb300_rotation(NULL, 0, 0, 0, prop, py, px);
	adda_gb300_polarizability(ADDA_POL_LDR, mre, mim, 2 * M_PI / dpl, gridspace, prop, py, 0, cc);
	for (int c = 0; c < 3; c++) cc_sqrt[0][c] = csqrt(cc[2 * c] + I * cc[2 * c + 1]);
	ref_index[0] = mre + I * mim; /* calculator.c:278: chi_inv = 4pi/(d^3 (m^2-1)) */
	for (int c = 0; c < 3; c++) chi_inv[0][c] = 4 * M_PI / (pow(gridspace, 3) * (ref_index[0] * ref_index[0] - 1));
	if (argc > 8 && !strcmp(argv[8], "wkb")) InitField = IF_WKB;
	if (argc > 9 && !strcmp(argv[8], "read")) {
		InitField = IF_READ;
		infi_fnameY = infi_fnameX = argv[9];
	}
	if (argc > 11 && !strcmp(argv[8], "chpoint")) { /* -chpoint <time> -chp_type <type> -chp_dir <dir> */
		chp_dir = argv[9];
		chp_type = !strcmp(argv[10], "normal") ? CHP_NORMAL : !strcmp(argv[10], "regular") ? CHP_REGULAR : CHP_ALWAYS;
		chp_time = atoi(argv[11]) > 0 ? atoi(argv[11]) : -1;
		if (argc > 12) maxiter = atoi(argv[12]);
	}
	if (argc > 11 && !strcmp(argv[8], "surf")) { /* -surf <h> <m_re> <m_im> -int_surf img */
		surface = true;
		hsub = atof(argv[9]);
		msub = atof(argv[10]) + I * atof(argv[11]);
		surfRCn = (1 - msub * msub) / (1 + msub * msub);
		ZsumShift = 2 * (hsub / gridspace - (boxZ - 1) / 2.0);
	}
	if (argc > 9 && !strcmp(argv[8], "chp_load")) {
		chp_dir = argv[9];
		load_chpoint = true;
	}
	time(&last_chp_wt);
	Einc = malloc(sizeof(doublecomplex) * local_nRows);
	xvec = malloc(sizeof(doublecomplex) * local_nRows);
	pvec = malloc(sizeof(doublecomplex) * local_nRows);
	if (surface) {
		double sc;
		if (adda_gb300_plane_wave_surf(local_nvoid_Ndip, position, boxX, boxY, boxZ, gridspace, WaveNum, prop, py, px,
				0, hsub, creal(msub), cimag(msub), 0, (double *)Einc, &sc)) return 4;
	}
	else adda_gb300_plane_wave(local_nvoid_Ndip, position, boxX, boxY, boxZ, gridspace, WaveNum, prop, py,
		(double *)Einc);
	InitDmatrix();
	int niter = IterativeSolver(method, INCPOL_Y);
	if (niter == -2) printf("mock host: exit after checkpoint\n"); /* CHP_EXIT: Calculator returns (calculator.c:312) */
	doublecomplex *y = malloc(sizeof(doublecomplex) * local_nRows);
	clock_t t = 0;
	ipr_required = true;
	double ip = 0;
	MatVec(Einc, y, &ip, false, &t, NULL);
	FILE *f = fopen(argv[7], "wb");
	long long n = (long long)local_nvoid_Ndip;
	fwrite(&n, sizeof(n), 1, f);
	fwrite(&niter, sizeof(niter), 1, f);
	fwrite(&ip, sizeof(ip), 1, f);
	fwrite(pvec, sizeof(doublecomplex), local_nRows, f);
	fwrite(y, sizeof(doublecomplex), local_nRows, f);
	if (surface) { /* the reference scatters through CalcFieldSurf in surface mode: no scattering output here */
		fclose(f);
		Free_FFT_Dmat();
		printf("mock host: %lld dipoles, %d iterations, %zu matvecs\n", n, niter, TotalMatVec);
		return 0;
	}
	/* scattered fields through the reference's CalcField call (wrapped at link time): forward and two more */
	const double dirs[3][3] = {{prop[0], prop[1], prop[2]}, {0.6, 0.0, 0.8}, {0.0, -1.0, 0.0}};
	for (int d = 0; d < 3; d++) {
		doublecomplex e[3];
		CalcField(e, dirs[d]);
		fwrite(e, sizeof(doublecomplex), 3, f);
	}
	/* the whole-solid-angle grid through the reference's CalcAlldir call (wrapped at link time): a small grid */
	double thv[5] = {180, 120, 90, 60, 0}, phv[4] = {0, 90, 180, 270};
	theta_int = (angle_set){0, 180, 5, thv};
	phi_int = (angle_set){0, 270, 4, phv};
	E_ad = malloc(sizeof(doublecomplex) * 2 * 20);
	E2_alldir = malloc(sizeof(double) * 20);
	CalcAlldir();
	fwrite(E2_alldir, sizeof(double), 20, f);
	/* three (theta, phi) pairs through the reference's CalcScatGrid call (wrapped at link time) */
	double sgt[3] = {30, 90, 150}, sgp[3] = {10, 200, 300};
	angles = (scat_grid_angles){SG_PAIRS, 3, {30, 150, 3, sgt}, {10, 300, 3, sgp}};
	EgridY = malloc(sizeof(doublecomplex) * 6);
	CalcScatGrid(INCPOL_Y);
	fwrite(EgridY, sizeof(doublecomplex), 6, f);
	fclose(f);
	Free_FFT_Dmat();
	printf("mock host: %lld dipoles, %d iterations, %zu matvecs\n", n, niter, TotalMatVec);
	return 0;
}
