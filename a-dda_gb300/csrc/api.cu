// api.cu - context management and the C-ABI entry points of include/adda_gb300.h.
#include "ctx.cuh"

#include <cstdio>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>

namespace adda {

static thread_local std::string g_err;

// largest L2 chunk budget the FP32 matvec tuner tries (MB)
constexpr int CHUNK_TUNE_MAX_MB = 128;
std::atomic<unsigned long long> g_launches{0};

void set_error(const std::string &msg) { g_err = msg; }

// exp(-2*pi*i*t/n) with octant reduction (arguments of cos/sin stay in [0, pi/4])
static void unit_root(long t, long n, double &c, double &s)
{
	t %= n;
	if (t < 0) t += n;
	const long e = 8 * t;
	const int oct = (int)(e / n);
	const double a = (double)(e - (long)oct * n) / (double)n * (M_PI / 4);
	const double ca = cos(a), sa = sin(a), cb = cos(M_PI / 4 - a), sb = sin(M_PI / 4 - a);
	double cc, ss;
	switch (oct) {
		case 0: cc = ca; ss = sa; break;
		case 1: cc = sb; ss = cb; break;
		case 2: cc = -sa; ss = ca; break;
		case 3: cc = -cb; ss = sb; break;
		case 4: cc = -ca; ss = -sa; break;
		case 5: cc = -sb; ss = -cb; break;
		case 6: cc = sa; ss = -ca; break;
		default: cc = cb; ss = -sb; break;
	}
	c = cc;
	s = -ss;
}

FftPlan make_plan(int n, int max_radix)
{
	FftPlan p;
	memset(&p, 0, sizeof(p));
	p.n = n;
	int m = n;
	while (m % max_radix == 0 && p.np < ADDA_FFT_MAXPASS) { p.r[p.np++] = max_radix; m /= max_radix; }
	for (int r = max_radix / 2; r >= 2; r /= 2)
		while (m % r == 0 && p.np < ADDA_FFT_MAXPASS) { p.r[p.np++] = r; m /= r; }
	const int odd[] = {3, 5, 7, 11, 13};
	for (int q : odd)
		while (m % q == 0 && p.np < ADDA_FFT_MAXPASS) { p.r[p.np++] = q; m /= q; }
	if (m != 1) p.np = -1; // unsupported factor
	return p;
}

} // namespace adda

using namespace adda;

extern "C" {

const char *adda_gb300_last_error(void) { return g_err.c_str(); }

double adda_gb300_last_solve_ms(const adda_gb300_ctx *c) { return c ? c->last_solve_ms : 0.0; }

uint64_t adda_gb300_kernel_launches(void) { return g_launches.load(); }

int adda_gb300_get_grid(const adda_gb300_ctx *c, int grid[3])
{
	if (!c || !grid) return ADDA_GB300_EINVAL;
	grid[0] = c->gX;
	grid[1] = c->gY;
	grid[2] = c->gZ;
	return ADDA_GB300_OK;
}

// n-th roots of unity of one axis. The FP32 table has a second part of n entries for the register FFT of the y
// transform (reg_fft, power-of-two n = T*E up to 512): W_n^(j1*k2) at k2*T + j1, so that the T lanes of a line read
// their step-1 twiddles from consecutive addresses.
static int upload_twiddles(adda_gb300_ctx *c, int which, int n)
{
	std::vector<double2> t64(n);
	std::vector<float2> t32(2 * (size_t)n, make_float2(0.f, 0.f));
	for (int t = 0; t < n; t++) {
		double cs, sn;
		unit_root(t, n, cs, sn);
		t64[t] = make_double2(cs, sn);
		t32[t] = make_float2((float)cs, (float)sn);
	}
	int T = 0;
	switch (n) {
		case 64: T = RegShape<64>::T; break;
		case 128: T = RegShape<128>::T; break;
		case 256: T = RegShape<256>::T; break;
		case 512: T = RegShape<512>::T; break;
		default: break;
	}
	for (int k2 = 0; T && k2 < n / T; k2++)
		for (int j1 = 0; j1 < T; j1++) t32[n + (size_t)k2 * T + j1] = t32[(size_t)j1 * k2 % n];
	ADDA_CUDA(cudaMalloc(&c->tw64[which], sizeof(double2) * n));
	ADDA_CUDA(cudaMalloc(&c->tw32[which], sizeof(float2) * 2 * (size_t)n));
	ADDA_CUDA(cudaMemcpy(c->tw64[which], t64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
	ADDA_CUDA(cudaMemcpy(c->tw32[which], t32.data(), sizeof(float2) * 2 * (size_t)n, cudaMemcpyHostToDevice));
	return ADDA_GB300_OK;
}

// one particle's lattice inside the context's box
struct Lat {
	size_t n;
	const uint16_t *pos;
	const uint8_t *mat;
};

static int create_impl(const adda_gb300_problem *p, adda_gb300_ctx *c, const std::vector<Lat> &lats)
{
	c->device = p->device;
	ADDA_CUDA(cudaSetDevice(p->device));
	ADDA_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
	ADDA_CUDA(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
	ADDA_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
	ADDA_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
	ADDA_CUDA(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming));
	ADDA_CUDA(cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming));
	c->bX = p->boxX; c->bY = p->boxY; c->bZ = p->boxZ;
	c->gX = p->gridX > 0 ? p->gridX : adda_gb300_fft_fit(2 * p->boxX, 1);
	c->gY = p->gridY > 0 ? p->gridY : adda_gb300_fft_fit(2 * p->boxY, 1);
	c->gZ = p->gridZ > 0 ? p->gridZ : adda_gb300_fft_fit(2 * p->boxZ, 2);
	if (c->gX < 2 * c->bX - 1 || c->gY < 2 * c->bY || c->gZ < 2 * c->bZ || c->gY % 2 || c->gZ % 2) {
		set_error("FFT grid must satisfy gridX >= 2*boxX-1 and even gridY >= 2*boxY, gridZ >= 2*boxZ");
		return ADDA_GB300_EINVAL;
	}
	c->DsY = c->gY / 2 + 1;
	c->DsZ = c->gZ / 2 + 1;
	c->P = (int)lats.size();
	c->N = 0;
	for (const Lat &l : lats) c->N = std::max(c->N, l.n);
	c->Rmax = p->nrhs_max > 0 ? p->nrhs_max : 1;
	if (c->P > 1 && (c->Rmax % c->P || p->surface)) {
		set_error("create_group: nrhs_max must be a multiple of the number of particles (and no substrate)");
		return ADDA_GB300_EINVAL;
	}
	c->rpp = c->Rmax / c->P;
	c->gridspace = p->gridspace;
	c->k = p->wavenum;
	if (p->interaction < ADDA_INT_POI || p->interaction > ADDA_INT_SO || !(p->nloc_rp >= 0)) {
		set_error("create: unknown interaction term or negative Gaussian width");
		return ADDA_GB300_EINVAL;
	}
	if (p->interaction == ADDA_INT_IGT_SO || p->interaction == ADDA_INT_SO) {
		if (!p->int_tables) {
			set_error("create: the igt_so and so interaction terms need the integral tables (problem.int_tables)");
			return ADDA_GB300_EINVAL;
		}
		c->int_tables.assign(p->int_tables, p->int_tables + ADDA_GB300_INT_TABLES);
		c->so_m = make_double2(p->so_m_re, p->so_m_im);
	}
	if ((p->interaction == ADDA_INT_FCD || p->interaction == ADDA_INT_FCD_ST) &&
		!(p->wavenum * p->gridspace < 3.14159265358979323846)) {
		set_error("create: the FCD interaction needs kd < pi (at least 2 dipoles per wavelength)");
		return ADDA_GB300_EINVAL;
	}
	c->interaction = p->interaction;
	c->nloc_rp = p->nloc_rp;
	if (p->surface) {
		if (p->refl < ADDA_REFL_IMG || p->refl > ADDA_REFL_HOST || (p->refl != ADDA_REFL_IMG && !p->refl_data) ||
			(p->msub_inf && p->refl != ADDA_REFL_IMG && p->refl != ADDA_REFL_HOST) || !std::isfinite(p->zsum_shift)) {
			set_error("create: surface mode needs a known reflection relation (with its data for SOM/HOST, image "
				"relation for a perfect reflector) and a finite zsum_shift");
			return ADDA_GB300_EINVAL;
		}
		c->surface = 1;
		c->refl = p->refl;
		c->msub_inf = p->msub_inf;
		c->msub = make_double2(p->msub_re, p->msub_im);
		c->zsum_shift = p->zsum_shift;
		const size_t nk = 2 * (size_t)c->bZ - 1;
		if (p->refl == ADDA_REFL_SOM) {
			const size_t n = nk * c->bY * c->bX * 4;
			c->refl_host.assign((const double2 *)p->refl_data, (const double2 *)p->refl_data + n);
		}
		else if (p->refl == ADDA_REFL_HOST) {
			const size_t n = nk * c->bY * (2 * (size_t)c->bX - 1) * 6;
			c->refl_host.assign((const double2 *)p->refl_data, (const double2 *)p->refl_data + n);
		}
	}
	const int g3[3] = {c->gX, c->gY, c->gZ};
	FftPlan *pl[3] = {c->px, c->py, c->pz};
	for (int d = 0; d < 3; d++) {
		pl[d][0] = make_plan(g3[d], 8);
		pl[d][1] = make_plan(g3[d], 16);
		if (pl[d][0].np < 0 || pl[d][1].np < 0) {
			set_error("FFT grid sizes must factor into 2,3,5,7,11,13");
			return ADDA_GB300_EINVAL;
		}
		int rc = upload_twiddles(c, d, g3[d]);
		if (rc) return rc;
	}
	// lattices: check order (z, y, x ascending), build per-line dipole ranges. Particle q of a group occupies slot q
	// of every lattice array: line starts [q][bZ*bY+1] (indices into its own dipoles), xy/material [q][N], positions
	// [q][N][3], N the largest particle (the other slots padded with zeros)
	const size_t N = c->N, nl = (size_t)c->bZ * c->bY + 1;
	c->pos.assign(3 * N * c->P, 0);
	c->mat.assign(N * c->P, 0);
	std::vector<uint32_t> ls(nl * c->P, 0), xy(std::max<size_t>(N * c->P, 1), 0);
	for (int q = 0; q < c->P; q++) {
		const Lat &L = lats[q];
		if (L.n && !L.pos) {
			set_error("create: a particle without positions");
			return ADDA_GB300_EINVAL;
		}
		std::copy(L.pos, L.pos + 3 * L.n, c->pos.begin() + 3 * N * q);
		if (L.mat) std::copy(L.mat, L.mat + L.n, c->mat.begin() + N * q);
		uint32_t *lq = ls.data() + nl * q;
		long prev = -1;
		for (size_t i = 0; i < L.n; i++) {
			const int x = L.pos[3 * i], y = L.pos[3 * i + 1], z = L.pos[3 * i + 2];
			if (x >= c->bX || y >= c->bY || z >= c->bZ) {
				set_error("dipole position outside the box");
				return ADDA_GB300_EINVAL;
			}
			const long key = ((long)z * c->bY + y) * c->bX + x;
			if (key <= prev) {
				set_error("dipole positions must be unique and sorted z-major, then y, then x");
				return ADDA_GB300_EINVAL;
			}
			prev = key;
			lq[(size_t)z * c->bY + y + 1]++;
			xy[N * q + i] = (uint32_t)x | ((uint32_t)y << 16);
		}
		for (size_t l = 1; l < nl; l++) lq[l] += lq[l - 1];
	}
	c->lat_stride = N;
	// the particle must lie entirely above the substrate (make_particle.c:2282): the lowest dipole layer zmin above
	// its own image, zsum_shift + 2*zmin > 0 (positions are z-major, so the first dipole is in the lowest layer)
	if (c->surface && N && !(c->zsum_shift + 2.0 * c->pos[2] > 0)) {
		set_error("create: the particle must be entirely above the substrate (zsum_shift + 2*zmin > 0)");
		return ADDA_GB300_EINVAL;
	}
	if (N > 0xffffffffu / 3) {
		set_error("too many dipoles");
		return ADDA_GB300_EINVAL;
	}
	const size_t NP = std::max<size_t>(N * c->P, 1);
	ADDA_CUDA(cudaMalloc(&c->d_line_start, sizeof(uint32_t) * ls.size()));
	ADDA_CUDA(cudaMalloc(&c->d_xy, sizeof(uint32_t) * NP));
	ADDA_CUDA(cudaMalloc(&c->d_mat, NP));
	ADDA_CUDA(cudaMalloc(&c->d_pos, sizeof(uint16_t) * 3 * NP));
	ADDA_CUDA(cudaMemcpy(c->d_line_start, ls.data(), sizeof(uint32_t) * ls.size(), cudaMemcpyHostToDevice));
	if (N) {
		ADDA_CUDA(cudaMemcpy(c->d_xy, xy.data(), sizeof(uint32_t) * N * c->P, cudaMemcpyHostToDevice));
		ADDA_CUDA(cudaMemcpy(c->d_mat, c->mat.data(), N * c->P, cudaMemcpyHostToDevice));
		ADDA_CUDA(cudaMemcpy(c->d_pos, c->pos.data(), sizeof(uint16_t) * 3 * N * c->P, cudaMemcpyHostToDevice));
	}
	// interaction matrix
	const size_t dlen = (size_t)c->gX * c->DsZ * c->DsY * 6;
	ADDA_CUDA(cudaMalloc(&c->D64, sizeof(double2) * dlen));
	ADDA_CUDA(cudaMalloc(&c->D32, sizeof(float2) * dlen));
	if (c->surface) {
		const size_t rlen = (size_t)c->gX * c->gZ * (c->gY / 2 + 1) * 6;
		ADDA_CUDA(cudaMalloc(&c->R64, sizeof(double2) * rlen));
		ADDA_CUDA(cudaMalloc(&c->R32, sizeof(float2) * rlen));
	}
	// matvec work: Xf for Rmax RHS in FP64; the z-chunk buffer is sized to ~48 MB so that it stays in L2
	const size_t R = c->Rmax;
	ADDA_CUDA(cudaMalloc(&c->Xf, sizeof(double2) * R * c->gX * 3 * (size_t)c->bZ * c->bY));
	const size_t slab = R * 3 * (size_t)c->gZ * c->bY; // complex elements of one x-slab for all RHS
	// FP64: 48 MB chunks. FP32: the chunk is tuned after the D matrix (tune_chunks) among budgets up to
	// CHUNK_TUNE_MAX_MB; ADDA_GB300_CHUNK_MB fixes the FP32 budget instead.
	const size_t budget = 48u << 20;
	c->CK64 = (int)std::max<size_t>(1, std::min<size_t>(c->gX, budget / (slab * sizeof(double2))));
	size_t b32 = budget;
	if (const char *e = getenv("ADDA_GB300_CHUNK_MB")) {
		const long mb = atol(e);
		if (mb > 0 && mb <= 4096) {
			b32 = (size_t)mb << 20;
			c->chunk_fixed = true;
		}
	}
	c->CK32 = (int)std::max<size_t>(1, std::min<size_t>(c->gX, b32 / (slab * sizeof(float2))));
	c->CK32max = c->chunk_fixed ? c->CK32
		: (int)std::max<size_t>(1, std::min<size_t>(c->gX, ((size_t)CHUNK_TUNE_MAX_MB << 20) / (slab * sizeof(float2))));
	const size_t tz = std::max(c->CK64 * sizeof(double2), c->CK32max * sizeof(float2)) * slab;
	ADDA_CUDA(cudaMalloc(&c->Tz, tz));
	ADDA_CUDA(cudaMalloc(&c->Tz2, tz));
	if (c->surface) {
		ADDA_CUDA(cudaMalloc(&c->TzR, tz));
		ADDA_CUDA(cudaMalloc(&c->TzR2, tz));
	}
	c->partial_len = (size_t)R * c->bY * c->bZ * 4; // K3 partial sums for the narrowest tile (one y-line per block)
	ADDA_CUDA(cudaMalloc(&c->partial, sizeof(double) * c->partial_len));
	ADDA_CUDA(cudaMalloc(&c->d_red, sizeof(double) * R * 4));
	ADDA_CUDA(cudaMalloc(&c->vin, sizeof(double2) * R * 3 * std::max<size_t>(N, 1)));
	ADDA_CUDA(cudaMalloc(&c->vout, sizeof(double2) * R * 3 * std::max<size_t>(N, 1)));
	if (c->P > 1) { // padded dipoles of smaller particles: the gather never writes them
		ADDA_CUDA(cudaMemset(c->vin, 0, sizeof(double2) * R * 3 * N));
		ADDA_CUDA(cudaMemset(c->vout, 0, sizeof(double2) * R * 3 * N));
	}
	c->cc_set.assign(R, 0);
	c->nmat = 0;
	int rc = matvec_setup(c);
	if (rc) return rc;
	// ADDA_GB300_FFT_SHAPE="w1,w2,pairs,nt" fixes the FP32 tile shape (no tuning of it)
	if (const char *e = getenv("ADDA_GB300_FFT_SHAPE")) {
		int v[4];
		if (sscanf(e, "%d,%d,%d,%d", v, v + 1, v + 2, v + 3) == 4 &&
			!matvec_set_shape(c, true, MvShape{v[0], v[1], v[2], v[3]}))
			c->shape_fixed = true;
	}
	return ADDA_GB300_OK;
}

int adda_gb300_destroy(adda_gb300_ctx *c)
{
	if (!c) return ADDA_GB300_OK;
	if (c->stream) cudaStreamSynchronize(c->stream);
	solver_free(c);
	void *bufs[] = {c->d_line_start, c->d_xy, c->d_mat, c->d_pos, c->D64, c->D32, c->cc64, c->ccs64, c->ccs32,
		c->Xf, c->Tz, c->TzR, c->Tz2, c->TzR2, c->R64, c->R32, c->partial, c->d_red, c->vin, c->vout, c->pvec64,
		c->tw64[0], c->tw64[1], c->tw64[2], c->tw32[0], c->tw32[1], c->tw32[2]};
	if (c->stream2) cudaStreamSynchronize(c->stream2);
	for (void *b : bufs)
		if (b) cudaFree(b);
	if (c->ev_fork) cudaEventDestroy(c->ev_fork);
	if (c->ev_join) cudaEventDestroy(c->ev_join);
	if (c->ev_in) cudaEventDestroy(c->ev_in);
	if (c->ev_out) cudaEventDestroy(c->ev_out);
	if (c->stream2) cudaStreamDestroy(c->stream2);
	if (c->stream) cudaStreamDestroy(c->stream);
	delete c;
	return ADDA_GB300_OK;
}

int adda_gb300_create(const adda_gb300_problem *p, adda_gb300_ctx **out)
{
	if (!p || !out || p->boxX < 1 || p->boxY < 1 || p->boxZ < 1 || (p->ndip && !p->position) ||
		p->boxX > 65535 || p->boxY > 65535 || p->boxZ > 65535 || !(p->gridspace > 0) || !(p->wavenum > 0)) {
		set_error("adda_gb300_create: invalid problem description");
		return ADDA_GB300_EINVAL;
	}
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device || p->device < 0) {
		cudaGetLastError();
		set_error("adda_gb300_create: no usable CUDA device");
		return ADDA_GB300_ECUDA;
	}
	adda_gb300_ctx *c = new adda_gb300_ctx();
	int rc = create_impl(p, c, {Lat{p->ndip, p->position, p->material}});
	if (rc) {
		std::string keep = g_err;
		adda_gb300_destroy(c);
		g_err = keep;
		return rc;
	}
	*out = c;
	return ADDA_GB300_OK;
}

int adda_gb300_create_group(const adda_gb300_problem *p, int nparticles, const size_t *ndip,
	const uint16_t *const *position, const uint8_t *const *material, adda_gb300_ctx **out)
{
	if (!p || !out || nparticles < 1 || !ndip || !position || p->boxX < 1 || p->boxY < 1 || p->boxZ < 1 ||
		p->boxX > 65535 || p->boxY > 65535 || p->boxZ > 65535 || !(p->gridspace > 0) || !(p->wavenum > 0)) {
		set_error("adda_gb300_create_group: invalid problem description");
		return ADDA_GB300_EINVAL;
	}
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device || p->device < 0) {
		cudaGetLastError();
		set_error("adda_gb300_create_group: no usable CUDA device");
		return ADDA_GB300_ECUDA;
	}
	std::vector<Lat> lats(nparticles);
	for (int q = 0; q < nparticles; q++) lats[q] = Lat{ndip[q], position[q], material ? material[q] : nullptr};
	adda_gb300_ctx *c = new adda_gb300_ctx();
	int rc = create_impl(p, c, lats);
	if (rc) {
		std::string keep = g_err;
		adda_gb300_destroy(c);
		g_err = keep;
		return rc;
	}
	*out = c;
	return ADDA_GB300_OK;
}

__global__ void fill_k(double2 *v, size_t n, unsigned seed);
__global__ void d2f_k(float2 *dst, const double2 *src, size_t n);

// The FP32 matvec's autotuner. The tile shape (threads per register-K2b block or (kz, RHS) pairs per generic-K2b
// block, y-lines per K2a/K2c and per K1/K3 block) sets occupancy and shared memory per block; the chunk (x-slabs whose z-transformed data pass through L2
// between K2a, K2b and K2c) trades L2 residency against launch count and tail waves; the best of both depends on
// the grid and the RHS count. Measured once per context on its own data sizes: the shape by coordinate descent over
// the alternatives the build holds (kept when 2 % faster), then balanced splits of the x-slabs into chunks of
// 24..CHUNK_TUNE_MAX_MB; one warm-up and two timed matvecs each with Rmax RHS of random data (CUDA events on the
// context stream). Runs from check_ready, i.e. only once the D matrix and the polarisability buffers a matvec reads
// exist, and before any graph capture. ADDA_GB300_CHUNK_MB / ADDA_GB300_FFT_SHAPE (or adda_gb300_set_fft_shape)
// fix either part.
static int tune_chunks(adda_gb300_ctx *c)
{
	if (c->chunk_tuned || c->N == 0 || !c->dready || !c->ccs32 || (c->chunk_fixed && c->shape_fixed))
		return ADDA_GB300_OK;
	ADDA_CUDA(cudaSetDevice(c->device));
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	ADDA_CUDA(cudaStreamIsCapturing(c->stream, &cap));
	if (cap != cudaStreamCaptureStatusNone) return ADDA_GB300_OK; // a caller is recording: keep the default
	c->chunk_tuned = true;
	const size_t slab = (size_t)c->Rmax * 3 * c->gZ * c->bY;
	const size_t n = (size_t)c->Rmax * 3 * c->N;
	fill_k<<<1024, 256, 0, c->stream>>>((double2 *)c->vin, n, 777u);
	ADDA_LAUNCHED();
	d2f_k<<<1024, 256, 0, c->stream>>>((float2 *)c->vout, (const double2 *)c->vin, n);
	ADDA_LAUNCHED();
	const float2 *in = (const float2 *)c->vout;
	float2 *out = (float2 *)c->vout + n;
	MvEpi e{EPI_NONE, nullptr, c->partial};
	cudaEvent_t e0, e1;
	ADDA_CUDA(cudaEventCreate(&e0));
	ADDA_CUDA(cudaEventCreate(&e1));
	int rc = ADDA_GB300_OK;
	// one warm-up and two timed FP32 matvecs of Rmax RHS with the current settings
	auto time_mv = [&](float &t) {
		if ((rc = matvec_run<float>(c, c->Rmax, in, out, 0, e, nullptr))) return false;
		cudaEventRecord(e0, c->stream);
		for (int i = 0; i < 2 && !rc; i++) rc = matvec_run<float>(c, c->Rmax, in, out, 0, e, nullptr);
		cudaEventRecord(e1, c->stream);
		if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = ADDA_GB300_ECUDA;
		if (rc) return false;
		cudaEventElapsedTime(&t, e0, e1);
		return true;
	};
	// 1. the tile shape, one dimension at a time over the alternatives the build holds (register-K2b threads per
	// block or generic-K2b pairs per block, then y-lines per K2a/K2c block, then per K1/K3 block), each kept when
	// faster; candidates that do not fit the axis lengths are skipped
	if (!c->shape_fixed) {
		float best = 1e30f;
		if (!time_mv(best)) goto done;
		for (int dim = 0; dim < 4; dim++) {
			static const int cand[4][3] = {{64, 128, 256}, {2, 4, 8}, {8, 16, 32}, {4, 8, 8}};
			for (int k = 0; k < 3; k++) {
				MvShape sh = c->shape[1], keep = sh;
				int &field = dim == 0 ? sh.nt : dim == 1 ? sh.pairs : dim == 2 ? sh.w2 : sh.w1;
				if (field == cand[dim][k] || (dim == 0 && !matvec_k2b_reg(c)) || (dim == 1 && matvec_k2b_reg(c)))
					continue;
				field = cand[dim][k];
				if (!matvec_shape_ok(c, true, sh)) continue;
				c->shape[1] = sh;
				float t = 0;
				if (!time_mv(t)) goto done;
				if (t < 0.98f * best) best = t;
				else c->shape[1] = keep;
			}
		}
	}
	// 2. the chunk: the gX x-slabs split into nc balanced chunks (no small tail chunk), from the largest chunk that
	// fits the Tz buffer down to about 24 MB
	if (!c->chunk_fixed) {
		int best_ck = c->CK32, last = -1;
		float best = 1e30f;
		const size_t min_ck = std::max<size_t>(1, ((size_t)24 << 20) / (slab * sizeof(float2)));
		for (int nc = 1; nc <= c->gX; nc++) {
			const int ck = (c->gX + nc - 1) / nc;
			if (ck > c->CK32max) continue;
			if (last > 0 && 5 * ck > 4 * last) continue; // next candidate at least 20 % smaller
			if ((size_t)ck < min_ck && last > 0) break;
			last = ck;
			c->CK32 = ck;
			float t = 0;
			if (!time_mv(t)) break;
			if (t < best) {
				best = t;
				best_ck = ck;
			}
		}
		c->CK32 = best_ck;
	}
done:
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

int adda_gb300_get_fft_shape(const adda_gb300_ctx *c, int prec, int shape[4])
{
	if (!c || !shape || (prec != ADDA_PREC_FP64 && prec != ADDA_PREC_FP32)) return ADDA_GB300_EINVAL;
	const MvShape &s = c->shape[prec == ADDA_PREC_FP32 ? 1 : 0];
	shape[0] = s.w1;
	shape[1] = s.w2;
	shape[2] = s.pairs;
	shape[3] = s.nt;
	return ADDA_GB300_OK;
}

int adda_gb300_get_l2_chunk(const adda_gb300_ctx *c, int prec)
{
	if (!c || (prec != ADDA_PREC_FP64 && prec != ADDA_PREC_FP32)) return ADDA_GB300_EINVAL;
	return prec == ADDA_PREC_FP32 ? c->CK32 : c->CK64;
}

int adda_gb300_set_fft_shape(adda_gb300_ctx *c, int prec, const int shape[4])
{
	if (!c || !shape || (prec != ADDA_PREC_FP64 && prec != ADDA_PREC_FP32)) {
		set_error("set_fft_shape: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	const bool f32 = prec == ADDA_PREC_FP32;
	int rc = matvec_set_shape(c, f32, MvShape{shape[0], shape[1], shape[2], f32 ? shape[3] : 128});
	if (!rc && f32) c->shape_fixed = true;
	return rc;
}

int adda_gb300_init_dmatrix(adda_gb300_ctx *c)
{
	if (!c) return ADDA_GB300_EINVAL;
	ADDA_CUDA(cudaSetDevice(c->device));
	return dmatrix_build(c);
}

size_t adda_gb300_dmatrix_len(const adda_gb300_ctx *c)
{
	return c ? (size_t)c->gX * c->DsZ * c->DsY * 6 : 0;
}

int adda_gb300_get_dmatrix(adda_gb300_ctx *c, double *out)
{
	if (!c || !out) return ADDA_GB300_EINVAL;
	if (!c->dready) {
		set_error("D matrix not initialised");
		return ADDA_GB300_ESTATE;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	ADDA_CUDA(cudaMemcpy(out, c->D64, sizeof(double2) * adda_gb300_dmatrix_len(c), cudaMemcpyDeviceToHost));
	return ADDA_GB300_OK;
}

size_t adda_gb300_rmatrix_len(const adda_gb300_ctx *c)
{
	return (c && c->surface) ? (size_t)c->gX * c->gZ * (c->gY / 2 + 1) * 6 : 0;
}

int adda_gb300_get_rmatrix(adda_gb300_ctx *c, double *out)
{
	if (!c || !out) return ADDA_GB300_EINVAL;
	if (!c->surface || !c->dready) {
		set_error("R matrix not initialised (no substrate, or adda_gb300_init_dmatrix not called)");
		return ADDA_GB300_ESTATE;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	ADDA_CUDA(cudaMemcpy(out, c->R64, sizeof(double2) * adda_gb300_rmatrix_len(c), cudaMemcpyDeviceToHost));
	return ADDA_GB300_OK;
}

__global__ void cc_sqrt_k(const double2 *cc, double2 *ccs64, float2 *ccs32, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
		// principal square root, as C99 csqrt (InitCC, calculator.c:273)
		const double a = cc[t].x, b = cc[t].y;
		const double m = hypot(a, b);
		double re = sqrt(0.5 * (m + fabs(a)));
		double im;
		if (re == 0) im = 0;
		else im = b / (2 * re);
		double2 r;
		if (a >= 0) r = make_double2(re, im);
		else r = make_double2(fabs(im), copysign(re, b));
		ccs64[t] = r;
		ccs32[t] = make_float2((float)r.x, (float)r.y);
	}
}

__global__ void cc_from_sqrt_k(double2 *cc, const double2 *ccs64, float2 *ccs32, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
		const double2 r = ccs64[t];
		cc[t] = make_double2(r.x * r.x - r.y * r.y, 2 * r.x * r.y);
		ccs32[t] = make_float2((float)r.x, (float)r.y);
	}
}

static int set_cc_impl(adda_gb300_ctx *c, int rhs, int per_dip, int nmat, const double *cc, bool given_sqrt = false)
{
	if (!c || !cc || rhs < 0 || rhs >= c->Rmax || (!per_dip && (nmat < 1 || nmat > 256))) {
		set_error("set_cc: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	if (!per_dip)
		for (size_t i = 0; i < c->mat.size(); i++)
			if (c->mat[i] >= nmat) {
				set_error("set_cc: a dipole's material index exceeds nmat");
				return ADDA_GB300_EINVAL;
			}
	ADDA_CUDA(cudaSetDevice(c->device));
	const size_t per = per_dip ? c->N * 3 : (size_t)nmat * 3;
	// (re)allocate when the mode or the table size changes; other RHS slots must then be set again
	const bool same = (c->cc64 && c->per_dip == per_dip && (per_dip || c->nmat == nmat));
	if (!same) {
		cudaFree(c->cc64); cudaFree(c->ccs64); cudaFree(c->ccs32);
		c->cc64 = c->ccs64 = nullptr;
		c->ccs32 = nullptr;
		ADDA_CUDA(cudaMalloc(&c->cc64, sizeof(double2) * per * c->Rmax));
		ADDA_CUDA(cudaMalloc(&c->ccs64, sizeof(double2) * per * c->Rmax));
		ADDA_CUDA(cudaMalloc(&c->ccs32, sizeof(float2) * per * c->Rmax));
		std::fill(c->cc_set.begin(), c->cc_set.end(), 0);
		c->per_dip = per_dip;
		c->nmat = per_dip ? 0 : nmat;
	}
	const int g = (int)std::min<size_t>((per + 255) / 256, 4096);
	if (given_sqrt) {
		ADDA_CUDA(cudaMemcpyAsync(c->ccs64 + per * rhs, cc, sizeof(double2) * per, cudaMemcpyHostToDevice, c->stream));
		cc_from_sqrt_k<<<g, 256, 0, c->stream>>>(c->cc64 + per * rhs, c->ccs64 + per * rhs, c->ccs32 + per * rhs, per);
	}
	else {
		ADDA_CUDA(cudaMemcpyAsync(c->cc64 + per * rhs, cc, sizeof(double2) * per, cudaMemcpyHostToDevice, c->stream));
		cc_sqrt_k<<<g, 256, 0, c->stream>>>(c->cc64 + per * rhs, c->ccs64 + per * rhs, c->ccs32 + per * rhs, per);
	}
	ADDA_LAUNCHED();
	ADDA_CUDA(cudaStreamSynchronize(c->stream));
	c->cc_set[rhs] = 1;
	return ADDA_GB300_OK;
}

int adda_gb300_set_cc(adda_gb300_ctx *c, int rhs, int nmat, const double *cc)
{
	return set_cc_impl(c, rhs, 0, nmat, cc);
}

int adda_gb300_set_cc_sqrt(adda_gb300_ctx *c, int rhs, int nmat, const double *cc_sqrt)
{
	return set_cc_impl(c, rhs, 0, nmat, cc_sqrt, true);
}

int adda_gb300_set_cc_dipole(adda_gb300_ctx *c, int rhs, const double *cc)
{
	return set_cc_impl(c, rhs, 1, 0, cc);
}

static int check_ready(adda_gb300_ctx *c, int nrhs)
{
	if (!c->dready) {
		set_error("D matrix not initialised (call adda_gb300_init_dmatrix)");
		return ADDA_GB300_ESTATE;
	}
	if (nrhs < 1 || nrhs > c->Rmax) {
		set_error("nrhs out of range");
		return ADDA_GB300_EINVAL;
	}
	for (int r = 0; r < nrhs; r++)
		if (!c->cc_set[r]) {
			set_error("polarisabilities not set for every RHS (call adda_gb300_set_cc)");
			return ADDA_GB300_ESTATE;
		}
	return tune_chunks(c);
}

__global__ void d2f_k(float2 *dst, const double2 *src, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
		dst[t] = make_float2((float)src[t].x, (float)src[t].y);
}

__global__ void f2d_k(double2 *dst, const float2 *src, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
		dst[t] = make_double2(src[t].x, src[t].y);
}

// the context's stream waits for the work queued on the caller's stream so far (inputs a caller filled there)
static int after_caller(adda_gb300_ctx *c)
{
	ADDA_CUDA(cudaEventRecord(c->ev_in, c->order));
	ADDA_CUDA(cudaStreamWaitEvent(c->stream, c->ev_in, 0));
	return ADDA_GB300_OK;
}

// the caller's stream waits for the work queued on the context's stream so far (results the caller reads there)
static int caller_after(adda_gb300_ctx *c)
{
	ADDA_CUDA(cudaEventRecord(c->ev_out, c->stream));
	ADDA_CUDA(cudaStreamWaitEvent(c->order, c->ev_out, 0));
	return ADDA_GB300_OK;
}

int adda_gb300_set_stream(adda_gb300_ctx *c, void *stream)
{
	if (!c) {
		set_error("set_stream: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	c->order = stream ? (cudaStream_t)stream : cudaStreamLegacy;
	return ADDA_GB300_OK;
}

int adda_gb300_matvec_device(adda_gb300_ctx *c, int prec, int nrhs, const void *d_arg, void *d_res, double *d_inprod,
	int her)
{
	if (!c || !d_arg || !d_res || (prec != ADDA_PREC_FP64 && prec != ADDA_PREC_FP32)) {
		set_error("matvec: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = check_ready(c, nrhs);
	if (rc) return rc;
	ADDA_CUDA(cudaSetDevice(c->device));
	if ((rc = after_caller(c))) return rc;
	const bool dbl = prec == ADDA_PREC_FP64;
	MvEpi e{d_inprod ? (int)EPI_NORM : (int)EPI_NONE, nullptr, c->partial};
	if (dbl) rc = matvec_run<double>(c, nrhs, (const double2 *)d_arg, (double2 *)d_res, her, e, nullptr);
	else rc = matvec_run<float>(c, nrhs, (const float2 *)d_arg, (float2 *)d_res, her, e, nullptr);
	if (rc) return rc;
	if (d_inprod) {
		const size_t nblk = matvec_partial_blocks(c, dbl);
		rc = reduce_partials(c, nrhs, c->partial, nblk, c->d_red);
		if (rc) return rc;
		ADDA_CUDA(cudaMemcpy2DAsync(d_inprod, sizeof(double), c->d_red, 4 * sizeof(double), sizeof(double), nrhs,
			cudaMemcpyDeviceToDevice, c->stream));
	}
	return caller_after(c);
}

int adda_gb300_matvec(adda_gb300_ctx *c, int prec, int nrhs, const double *argvec, double *resultvec, double *inprod,
	int her)
{
	if (!c || !argvec || !resultvec) {
		set_error("matvec: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = check_ready(c, nrhs);
	if (rc) return rc;
	ADDA_CUDA(cudaSetDevice(c->device));
	const size_t n = (size_t)nrhs * 3 * c->N;
	// group contexts: the gather writes only real dipoles, so the padding of the result comes back as zeros
	if (c->P > 1) ADDA_CUDA(cudaMemsetAsync(c->vout, 0, sizeof(double2) * n, c->stream));
	if (prec == ADDA_PREC_FP64) {
		ADDA_CUDA(cudaMemcpyAsync(c->vin, argvec, sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
		MvEpi e{inprod ? (int)EPI_NORM : (int)EPI_NONE, nullptr, c->partial};
		rc = matvec_run<double>(c, nrhs, (const double2 *)c->vin, (double2 *)c->vout, her, e, nullptr);
		if (rc) return rc;
		ADDA_CUDA(cudaMemcpyAsync(resultvec, c->vout, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
	}
	else if (prec == ADDA_PREC_FP32) {
		// stage the double host vector, round it on the device, compute, widen the result back (vout holds the 2n
		// float2 of the rounded input and the FP32 result: n double2)
		double2 *din = (double2 *)c->vin;
		float2 *fin = (float2 *)c->vout, *fout = (float2 *)c->vout + n;
		ADDA_CUDA(cudaMemcpyAsync(din, argvec, sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
		d2f_k<<<(int)std::min<size_t>((n + 255) / 256, 8192), 256, 0, c->stream>>>(fin, din, n);
		ADDA_LAUNCHED();
		MvEpi e{inprod ? (int)EPI_NORM : (int)EPI_NONE, nullptr, c->partial};
		rc = matvec_run<float>(c, nrhs, fin, fout, her, e, nullptr);
		if (rc) return rc;
		f2d_k<<<(int)std::min<size_t>((n + 255) / 256, 8192), 256, 0, c->stream>>>(din, fout, n);
		ADDA_LAUNCHED();
		ADDA_CUDA(cudaMemcpyAsync(resultvec, din, sizeof(double2) * n, cudaMemcpyDeviceToHost, c->stream));
	}
	else {
		set_error("matvec: prec must be ADDA_PREC_FP64 or ADDA_PREC_FP32");
		return ADDA_GB300_EINVAL;
	}
	if (inprod) {
		const size_t nblk = matvec_partial_blocks(c, prec == ADDA_PREC_FP64);
		rc = reduce_partials(c, nrhs, c->partial, nblk, c->d_red);
		if (rc) return rc;
		std::vector<double> red(4 * (size_t)nrhs);
		ADDA_CUDA(cudaMemcpyAsync(red.data(), c->d_red, sizeof(double) * 4 * nrhs, cudaMemcpyDeviceToHost,
			c->stream));
		ADDA_CUDA(cudaStreamSynchronize(c->stream));
		for (int r = 0; r < nrhs; r++) inprod[r] = red[4 * r];
	}
	ADDA_CUDA(cudaStreamSynchronize(c->stream));
	return ADDA_GB300_OK;
}

int adda_gb300_solve(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int nrhs, const double *einc,
	double *xvec, double *pvec, adda_gb300_rhs_stats *stats, double *resid_hist, int hist_cap)
{
	if (!c || !sp || !einc) {
		set_error("solve: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = check_ready(c, nrhs);
	if (rc) return rc;
	ADDA_CUDA(cudaSetDevice(c->device));
	return solver_solve(c, sp, nrhs, einc, xvec, pvec, stats, resid_hist, hist_cap);
}

size_t adda_gb300_chpoint_size(const adda_gb300_ctx *c, int method)
{
	return c ? solver_chpoint_size(c, method) : 0;
}

int adda_gb300_chpoint_save(adda_gb300_ctx *c, int rhs, void *buf, size_t size)
{
	if (c && c->P > 1) {
		set_error("chpoint_save: checkpoints hold one particle's vectors (not a group context)");
		return ADDA_GB300_ESTATE;
	}
	if (!c) {
		set_error("chpoint_save: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return solver_chpoint_save(c, rhs, buf, size);
}

int adda_gb300_chpoint_load(adda_gb300_ctx *c, int rhs, const void *buf, size_t size)
{
	if (c && c->P > 1) {
		set_error("chpoint_load: checkpoints hold one particle's vectors (not a group context)");
		return ADDA_GB300_ESTATE;
	}
	if (!c) {
		set_error("chpoint_load: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return solver_chpoint_load(c, rhs, buf, size);
}

int adda_gb300_solve_many(int nctx, adda_gb300_ctx *const *ctxs, const adda_gb300_solve_params *sp, const int *nrhs,
	const double *const *einc, double *const *xvec, double *const *pvec, adda_gb300_rhs_stats *const *stats)
{
	if (nctx < 0 || (nctx && (!ctxs || !sp || !nrhs || !einc))) {
		set_error("solve_many: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	std::vector<int> rcs(nctx, ADDA_GB300_OK);
	std::vector<std::string> errs(nctx);
	std::vector<std::thread> th;
	th.reserve(nctx);
	for (int i = 0; i < nctx; i++)
		th.emplace_back([&, i]() {
			rcs[i] = adda_gb300_solve(ctxs[i], sp, nrhs[i], einc[i], xvec ? xvec[i] : nullptr,
				pvec ? pvec[i] : nullptr, stats ? stats[i] : nullptr, nullptr, 0);
			if (rcs[i]) errs[i] = g_err;
		});
	for (auto &t : th) t.join();
	for (int i = 0; i < nctx; i++)
		if (rcs[i]) {
			set_error("solve_many: context " + std::to_string(i) + ": " + errs[i]);
			return rcs[i];
		}
	return ADDA_GB300_OK;
}

int adda_gb300_solve_device(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int nrhs, const void *d_einc,
	void *d_xvec, void *d_pvec, adda_gb300_rhs_stats *stats)
{
	if (!c || !sp || !d_einc) {
		set_error("solve_device: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = check_ready(c, nrhs);
	if (rc) return rc;
	ADDA_CUDA(cudaSetDevice(c->device));
	if ((rc = after_caller(c))) return rc;
	return solver_solve_dev(c, sp, nrhs, (const double2 *)d_einc, (double2 *)d_xvec, (double2 *)d_pvec, stats);
}

__global__ void fill_k(double2 *v, size_t n, unsigned seed)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
		unsigned h = (unsigned)(t * 2654435761u) ^ seed;
		h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
		unsigned g = h * 0x27d4eb2du; g ^= g >> 16;
		v[t] = make_double2((h & 0xffffff) / 16777216.0 - 0.5, (g & 0xffffff) / 16777216.0 - 0.5);
	}
}

__global__ void flush_k(float4 *buf, size_t n, float v)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
		buf[t] = make_float4(v, v, v, v);
}

int adda_gb300_time_matvec(adda_gb300_ctx *c, int prec, int nrhs, int iters, size_t flush_bytes, double *ms)
{
	if (!c || !ms || iters < 1 || (prec != ADDA_PREC_FP64 && prec != ADDA_PREC_FP32)) {
		set_error("time_matvec: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	int rc = check_ready(c, nrhs);
	if (rc) return rc;
	ADDA_CUDA(cudaSetDevice(c->device));
	const size_t n = (size_t)nrhs * 3 * c->N;
	const bool dbl = prec == ADDA_PREC_FP64;
	fill_k<<<1024, 256, 0, c->stream>>>((double2 *)c->vin, n, 12345u);
	ADDA_LAUNCHED();
	if (!dbl) {
		d2f_k<<<1024, 256, 0, c->stream>>>((float2 *)c->vout, (const double2 *)c->vin, n);
		ADDA_LAUNCHED();
	}
	const void *in = dbl ? c->vin : c->vout;
	void *out = dbl ? c->vout : (void *)((float2 *)c->vout + n);
	float4 *fl = nullptr;
	const size_t nfl = flush_bytes / sizeof(float4);
	if (nfl) ADDA_CUDA(cudaMalloc(&fl, nfl * sizeof(float4)));
	MvEpi e{EPI_NONE, nullptr, c->partial};
	cudaEvent_t e0, e1;
	ADDA_CUDA(cudaEventCreate(&e0));
	ADDA_CUDA(cudaEventCreate(&e1));
	double total = 0;
	for (int it = -1; it < iters && !rc; it++) {
		if (nfl) {
			flush_k<<<1024, 256, 0, c->stream>>>(fl, nfl, (float)it);
			count_launch();
		}
		cudaEventRecord(e0, c->stream);
		rc = dbl ? matvec_run<double>(c, nrhs, (const double2 *)in, (double2 *)out, 0, e, nullptr)
			: matvec_run<float>(c, nrhs, (const float2 *)in, (float2 *)out, 0, e, nullptr);
		cudaEventRecord(e1, c->stream);
		cudaEventSynchronize(e1);
		float t = 0;
		cudaEventElapsedTime(&t, e0, e1);
		if (it >= 0) total += t;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (fl) cudaFree(fl);
	if (rc) return rc;
	ADDA_CUDA(cudaGetLastError());
	*ms = total / iters;
	return ADDA_GB300_OK;
}

int adda_gb300_vjp_chi(adda_gb300_ctx *c, const adda_gb300_solve_params *sp, int rhs, const double prop[3],
	const double incpol[3], const double *dinv_alpha, double *grad_cext, double *grad_cabs)
{
	if (c && c->surface) {
		set_error("vjp_chi: free-space formula; in surface mode the reference scatters through CalcFieldSurf "
			"(crosssec.c:601-800), which is not provided (Cext/Cabs: adda_gb300_cross_sections_beam)");
		return ADDA_GB300_ESTATE;
	}
	if (c && c->P > 1) {
		set_error("vjp_chi: one particle per context (not a group context)");
		return ADDA_GB300_ESTATE;
	}
	if (!c || !sp || !prop || !incpol || !dinv_alpha || !grad_cext || !grad_cabs) {
		set_error("vjp_chi: invalid arguments");
		return ADDA_GB300_EINVAL;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return vjp_chi(c, sp, rhs, prop, incpol, dinv_alpha, grad_cext, grad_cabs);
}

int adda_gb300_cross_sections(adda_gb300_ctx *c, int nrhs, const double *prop, const double *incpol, double *cext,
	double *cabs)
{
	if (c && c->surface) {
		set_error("cross_sections: free-space formula; in surface mode the reference scatters through CalcFieldSurf "
			"(crosssec.c:601-800), which is not provided (Cext/Cabs: adda_gb300_cross_sections_beam)");
		return ADDA_GB300_ESTATE;
	}
	if (!c || !prop || !incpol || nrhs < 1 || nrhs > c->last_nrhs || !c->pvec64) {
		set_error("cross_sections: no solution available for that many RHS");
		return ADDA_GB300_ESTATE;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return cross_sections(c, nrhs, prop, incpol, cext, cabs);
}

int adda_gb300_cross_sections_beam(adda_gb300_ctx *c, int nrhs, const double *einc, double inc_scale, double *cext,
	double *cabs)
{
	if (!c || !einc || nrhs < 1 || nrhs > c->last_nrhs || !c->pvec64 || !(inc_scale > 0)) {
		set_error("cross_sections_beam: no solution available for that many RHS, or invalid arguments");
		return ADDA_GB300_ESTATE;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return cross_sections_beam(c, nrhs, einc, inc_scale, cext, cabs);
}

int adda_gb300_scattering_integrals(adda_gb300_ctx *c, int nrhs, const adda_gb300_integr_parms p[2],
	const double prop[3], const double incpolx[3], const double incpoly[3], double *csca, double *csca_g)
{
	if (c && c->surface) {
		set_error("scattering_integrals: free-space formula; in surface mode the reference scatters through CalcFieldSurf "
			"(crosssec.c:601-800), which is not provided (Cext/Cabs: adda_gb300_cross_sections_beam)");
		return ADDA_GB300_ESTATE;
	}
	if (!c || !p || !prop || !incpolx || !incpoly || !csca || !csca_g || nrhs < 1 || nrhs > c->last_nrhs ||
		!c->pvec64) {
		set_error("scattering_integrals: invalid arguments or no solution available for that many RHS");
		return ADDA_GB300_ESTATE;
	}
	const int nth = adda_gb300_integr_points(&p[0], 1, nullptr), nph = adda_gb300_integr_points(&p[1], 0, nullptr);
	if (nth < 1 || nph < 1) {
		set_error("scattering_integrals: inconsistent integration parameters");
		return ADDA_GB300_EINVAL;
	}
	std::vector<double> th(nth), ph(nph), dirs((size_t)nth * nph * 3);
	adda_gb300_integr_points(&p[0], 1, th.data());
	adda_gb300_integr_points(&p[1], 0, ph.data());
	const double d2r = 0.017453292519943295769236907684886;
	for (int i = 0; i < nth; i++) {
		const double t = d2r * th[i], ct = cos(t), st = sin(t);
		for (int j = 0; j < nph; j++) {
			const double f = d2r * ph[j], cf = cos(f), sf = sin(f);
			double *d = &dirs[((size_t)i * nph + j) * 3];
			for (int a = 0; a < 3; a++) d[a] = ct * prop[a] + st * (cf * incpolx[a] + sf * incpoly[a]);
		}
	}
	const size_t nd = (size_t)nth * nph;
	std::vector<double> e((size_t)nrhs * nd * 6);
	ADDA_CUDA(cudaSetDevice(c->device));
	int rc = scattered_fields(c, nrhs, (int)nd, dirs.data(), e.data());
	if (rc) return rc;
	std::vector<double> v(nd);
	const double k2 = c->k * c->k, four_pi = 12.566370614359172953850573533118;
	for (int r = 0; r < nrhs; r++) {
		std::vector<double> e2(nd);
		for (size_t q = 0; q < nd; q++) {
			const double *x = &e[((size_t)r * nd + q) * 6];
			e2[q] = x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3] + x[4] * x[4] + x[5] * x[5];
		}
		double res;
		adda_gb300_romberg2d(p, 1, e2.data(), &res); // ScaCross
		csca[r] = res * four_pi / k2;
		for (int comp = 0; comp < 3; comp++) { // gx, gy, gz integrands (crosssec.c:1172-1245)
			for (int i = 0; i < nth; i++) {
				const double t = d2r * th[i];
				for (int j = 0; j < nph; j++) {
					const size_t q = (size_t)i * nph + j;
					if (comp == 2) v[q] = e2[q] * cos(t);
					else if (th[i] == 180) v[q] = 0;
					else v[q] = e2[q] * sin(t) * (comp ? sin(d2r * ph[j]) : cos(d2r * ph[j]));
				}
			}
			adda_gb300_romberg2d(p, 1, v.data(), &res);
			csca_g[3 * r + comp] = res * four_pi / k2;
		}
	}
	return ADDA_GB300_OK;
}

int adda_gb300_scattered_fields(adda_gb300_ctx *c, int nrhs, int ndir, const double *dirs, double *ebuff)
{
	if (c && c->surface) {
		set_error("scattered_fields: free-space formula; in surface mode the reference scatters through CalcFieldSurf "
			"(crosssec.c:601-800), which is not provided (Cext/Cabs: adda_gb300_cross_sections_beam)");
		return ADDA_GB300_ESTATE;
	}
	if (!c || !dirs || !ebuff || ndir < 1 || nrhs < 1 || nrhs > c->last_nrhs || !c->pvec64) {
		set_error("scattered_fields: invalid arguments or no solution available for that many RHS");
		return ADDA_GB300_ESTATE;
	}
	ADDA_CUDA(cudaSetDevice(c->device));
	return scattered_fields(c, nrhs, ndir, dirs, ebuff);
}

} // extern "C"
