// matvec.cu - the FFT-accelerated DDA matrix-vector product y = x + S.D.S.x on the GPU (MatVec, src/matvec.c:128).
//
// Data flow for R right-hand sides sharing one interaction matrix D (all in HBM unless noted):
//   K1 mv_scatter_fftx : per (rhs, z, block of W y-lines): gather S.x of the dipoles of those x-lines straight from
//                        the dipole vector (no zeroed expanded grid, the reference's Xmatrix fill + Arith1), pad to
//                        gridX in shared memory, forward FFT along x  ->  Xf[r][kx][comp][z][y]
//   then per chunk of CK x-slabs (chunk buffer Tz sized to stay in L2):
//   K2a mv_fftz        : forward FFT along z of each y-line block (zero padding z>=boxZ in shared memory)
//   K2b mv_fft_y_dmul  : per (kx, kz block): forward FFT along y, 6-component symmetric D~ x X~ product for all RHS at
//                        once (D read once per grid point and reused by every RHS), inverse FFT along y
//   K2c mv_fftz (inv)  : inverse FFT along z, keep z<boxZ  ->  Xf
//   K3 mv_fftx_gather  : inverse FFT along x, y = x + S.X for the dipoles of the lines, optional Krylov reductions
//                        (|y|^2, x.y, y.u*, x.y*) as deterministic per-block partial sums.
// The reference's explicit transposes (TransposeYZ), slice zeroing and copies (Arith2/Arith4) do not exist here:
// every tile is loaded along the contiguous axis of its buffer and transformed in element-major shared memory.
#include "ctx.cuh"

#include <algorithm>

namespace adda {

namespace {

// T = arithmetic of the FFTs, D and the expanded grid (float or double); V = complex type of the dipole vectors the
// caller passes (float2 or double2). With T=float, V=double2 (the MIXED solver) the inputs are rounded on the fly and
// y = x + S.X is accumulated in double, so the identity part of A is exact.
template <typename T, typename V> struct MvP {
	typedef typename CxT<T>::type C;
	int bX, bY, bZ, gX, gY, gZ, DsY, DsZ;
	int R;
	size_t N;
	const uint32_t *line_start;
	const uint32_t *xy;
	const uint8_t *mat;
	const C *ccs;   // per-RHS cc_sqrt: [R][nmat][3] or [R][N][3]
	int nmat, per_dip;
	const V *arg;
	V *res;
	C *Xf;
	C *Tz;
	int CK, kx0;
	const C *D;
	FftPlan px, py, pz;
	const C *twx, *twy, *twz;
	int her;
	const int *done; // per-RHS done flags (may be null): every kernel returns at once when all are set
};

template <typename To, typename From> __device__ __forceinline__ To cvt(From a) { return from_d2<To>(to_d2(a)); }

template <typename P> __device__ __forceinline__ bool all_done(const P &p)
{
	if (!p.done) return false;
	for (int r = 0; r < p.R; r++)
		if (!p.done[r]) return false;
	return true;
}

template <typename C> __device__ __forceinline__ C ccs_of(const C *ccs, int per_dip, int nmat, size_t N, int r,
	size_t i, uint8_t m, int comp)
{
	return per_dip ? ccs[((size_t)r * N + i) * 3 + comp] : ccs[((size_t)r * nmat + m) * 3 + comp];
}

// K1: scatter S.x of W consecutive x-lines (one z) into shared memory and FFT along x. Tile: gX x (3*W) lines.
template <typename T, typename V, int W> __global__ void __launch_bounds__(256) mv_scatter_fftx(MvP<T, V> p)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	constexpr int nl = 3 * W, LS = tile_ls(3 * W);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)p.gX * LS;
	const int r = blockIdx.z, z = blockIdx.y, y0 = blockIdx.x * W;
	const int wy = min(W, p.bY - y0);
	for (int t = threadIdx.x; t < p.gX * LS; t += blockDim.x) a[t] = cx<C>(0, 0);
	__syncthreads();
	const size_t line = (size_t)z * p.bY + y0;
	const uint32_t i0 = p.line_start[line], i1 = p.line_start[line + wy];
	const V *arg = p.arg + (size_t)r * p.N * 3;
	for (uint32_t t = threadIdx.x; t < (i1 - i0) * 3; t += blockDim.x) {
		const size_t i = i0 + t / 3;
		const int comp = t % 3;
		const uint32_t q = p.xy[i];
		const int x = q & 0xffff, y = q >> 16;
		C v = cvt<C>(arg[i * 3 + comp]);
		if (p.her) v = cconj(v);
		v = cmul(ccs_of(p.ccs, p.per_dip, p.nmat, p.N, r, i, p.mat[i], comp), v);
		a[x * LS + comp * W + (y - y0)] = v;
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p.px, nl, LS, p.twx, false);
	const size_t plane = (size_t)p.bZ * p.bY;
	for (int t = threadIdx.x; t < p.gX * 3 * wy; t += blockDim.x) {
		const int yy = t % wy, rest = t / wy;
		const int comp = rest % 3, kx = rest / 3;
		p.Xf[(((size_t)r * p.gX + kx) * 3 + comp) * plane + (size_t)z * p.bY + y0 + yy] = o[kx * LS + comp * W + yy];
	}
}

// K2a/K2c: FFT along z of W consecutive y-lines of one (rhs, kx, comp). Forward reads Xf (z<bZ, zero padded) and
// writes Tz (all kz); inverse reads Tz and writes z<bZ back to Xf.
template <typename T, typename V, int W, bool INV> __global__ void __launch_bounds__(256) mv_fftz(MvP<T, V> p)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	constexpr int LS = tile_ls(W);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)p.gZ * LS;
	const int r = blockIdx.z;
	const int kxl = blockIdx.y / 3, comp = blockIdx.y % 3;
	const int kx = p.kx0 + kxl;
	const int y0 = blockIdx.x * W;
	const int wy = min(W, p.bY - y0);
	const size_t plane = (size_t)p.bZ * p.bY;
	C *xf = p.Xf + (((size_t)r * p.gX + kx) * 3 + comp) * plane + y0;
	C *tz = p.Tz + (((size_t)r * p.CK + kxl) * 3 + comp) * (size_t)p.gZ * p.bY + y0;
	if (!INV) {
		for (int t = threadIdx.x; t < p.gZ * W; t += blockDim.x) {
			const int yy = t % W, z = t / W;
			a[z * LS + yy] = (z < p.bZ && yy < wy) ? xf[(size_t)z * p.bY + yy] : cx<C>(0, 0);
		}
	}
	else {
		for (int t = threadIdx.x; t < p.gZ * W; t += blockDim.x) {
			const int yy = t % W, z = t / W;
			a[z * LS + yy] = (yy < wy) ? tz[(size_t)z * p.bY + yy] : cx<C>(0, 0);
		}
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p.pz, W, LS, p.twz, INV);
	if (!INV) {
		for (int t = threadIdx.x; t < p.gZ * wy; t += blockDim.x) {
			const int yy = t % wy, z = t / wy;
			tz[(size_t)z * p.bY + yy] = o[z * LS + yy];
		}
	}
	else {
		for (int t = threadIdx.x; t < p.bZ * wy; t += blockDim.x) {
			const int yy = t % wy, z = t / wy;
			xf[(size_t)z * p.bY + yy] = o[z * LS + yy];
		}
	}
}

// K2b: per (kx, block of KB kz, group of RG RHS): y-FFT, D product (matvec.c:271-305 incl. reduced-FFT signs),
// inverse y-FFT. Lines l = (rr*3 + comp)*KB + kk, rr = RHS within the group.
template <typename T, typename V> __global__ void __launch_bounds__(256) mv_fft_y_dmul(MvP<T, V> p, int KB, int RG)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	C *a = reinterpret_cast<C *>(smem_raw);
	const int rg0 = blockIdx.z * RG;
	const int rgn = min(RG, p.R - rg0);
	const int nl = RG * 3 * KB;
	const int LS = tile_ls(nl);
	C *b = a + (size_t)p.gY * LS;
	const int kxl = blockIdx.y, kx = p.kx0 + kxl;
	const int kz0 = blockIdx.x * KB;
	const size_t lz = (size_t)p.gZ * p.bY; // one (rhs, kx, comp) block of Tz
	for (int t = threadIdx.x; t < nl * p.gY; t += blockDim.x) {
		const int y = t % p.gY, l = t / p.gY;
		const int kk = l % KB, rc = l / KB;
		const int rr = rc / 3, comp = rc % 3;
		const int kz = kz0 + kk;
		C v = cx<C>(0, 0);
		if (y < p.bY && kz < p.gZ && rr < rgn)
			v = p.Tz[(((size_t)(rg0 + rr) * p.CK + kxl) * 3 + comp) * lz + (size_t)kz * p.bY + y];
		a[y * LS + l] = v;
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p.py, nl, LS, p.twy, false);
	C *s = (o == a) ? b : a;
	for (int t = threadIdx.x; t < KB * p.gY; t += blockDim.x) {
		const int ky = t % p.gY, kk = t / p.gY;
		const int kz = kz0 + kk;
		if (kz >= p.gZ) continue;
		const bool ry = ky >= p.DsY, rz = kz >= p.DsZ;
		const int yy = ry ? p.gY - ky : ky, zz = rz ? p.gZ - kz : kz;
		const C *f = p.D + (((size_t)kx * p.DsZ + zz) * p.DsY + yy) * 6;
		C m0 = f[0], m1 = f[1], m2 = f[2], m3 = f[3], m4 = f[4], m5 = f[5];
		if (ry) {
			m1 = cneg(m1);
			if (rz) m2 = cneg(m2);
			else m4 = cneg(m4);
		}
		else if (rz) {
			m2 = cneg(m2);
			m4 = cneg(m4);
		}
		for (int rr = 0; rr < rgn; rr++) {
			const int l0 = (rr * 3 + 0) * KB + kk, l1 = (rr * 3 + 1) * KB + kk, l2 = (rr * 3 + 2) * KB + kk;
			const C v0 = o[ky * LS + l0], v1 = o[ky * LS + l1], v2 = o[ky * LS + l2];
			o[ky * LS + l0] = cfma(m0, v0, cfma(m1, v1, cmul(m2, v2)));
			o[ky * LS + l1] = cfma(m1, v0, cfma(m3, v1, cmul(m4, v2)));
			o[ky * LS + l2] = cfma(m2, v0, cfma(m4, v1, cmul(m5, v2)));
		}
	}
	__syncthreads();
	C *o2 = fft_tile<C>(o, s, p.py, nl, LS, p.twy, true);
	for (int t = threadIdx.x; t < nl * p.bY; t += blockDim.x) {
		const int y = t % p.bY, l = t / p.bY;
		const int kk = l % KB, rc = l / KB;
		const int rr = rc / 3, comp = rc % 3;
		const int kz = kz0 + kk;
		if (kz < p.gZ && rr < rgn)
			p.Tz[(((size_t)(rg0 + rr) * p.CK + kxl) * 3 + comp) * lz + (size_t)kz * p.bY + y] = o2[y * LS + l];
	}
}

template <typename T> __device__ __forceinline__ double block_sum(double v, double *sh)
{
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	__syncthreads();
	if (lane == 0) sh[wid] = v;
	__syncthreads();
	double s = 0;
	if (threadIdx.x == 0)
		for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
	return s; // valid in thread 0
}

// K3: inverse FFT along x of W y-lines (one z), then y = x + S.X for their dipoles, with the epilogue reductions.
template <typename T, typename V, int W>
__global__ void __launch_bounds__(256) mv_fftx_gather(MvP<T, V> p, MvEpi e)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ double red[32];
	if (all_done(p)) return;
	constexpr int nl = 3 * W, LS = tile_ls(3 * W);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)p.gX * LS;
	const int r = blockIdx.z, z = blockIdx.y, y0 = blockIdx.x * W;
	const int wy = min(W, p.bY - y0);
	const size_t plane = (size_t)p.bZ * p.bY;
	for (int t = threadIdx.x; t < p.gX * nl; t += blockDim.x) {
		const int yy = t % W, rest = t / W;
		const int comp = rest % 3, kx = rest / 3;
		a[kx * LS + comp * W + yy] = (yy < wy)
			? p.Xf[(((size_t)r * p.gX + kx) * 3 + comp) * plane + (size_t)z * p.bY + y0 + yy]
			: cx<C>(0, 0);
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p.px, nl, LS, p.twx, true);
	const size_t line = (size_t)z * p.bY + y0;
	const uint32_t i0 = p.line_start[line], i1 = p.line_start[line + wy];
	const V *arg = p.arg + (size_t)r * p.N * 3;
	V *res = p.res + (size_t)r * p.N * 3;
	const V *u = e.u ? reinterpret_cast<const V *>(e.u) + (size_t)r * p.N * 3 : nullptr;
	double s0 = 0, s1r = 0, s1i = 0;
	for (uint32_t t = threadIdx.x; t < (i1 - i0) * 3; t += blockDim.x) {
		const size_t i = i0 + t / 3;
		const int comp = t % 3;
		const uint32_t q = p.xy[i];
		const int x = q & 0xffff, y = q >> 16;
		V xv = arg[i * 3 + comp];
		if (p.her) xv = cconj(xv);
		const C sx = cmul(ccs_of(p.ccs, p.per_dip, p.nmat, p.N, r, i, p.mat[i], comp), o[x * LS + comp * W + (y - y0)]);
		V yv = cadd(xv, cvt<V>(sx));
		if (p.her) yv = cconj(yv);
		res[i * 3 + comp] = yv;
		if (e.mode) {
			const double2 y2 = to_d2(yv);
			if (e.mode & EPI_NORM) s0 += y2.x * y2.x + y2.y * y2.y;
			if (e.mode & EPI_DOT_ARG) {
				const double2 x2 = to_d2(arg[i * 3 + comp]);
				s1r += x2.x * y2.x - x2.y * y2.y;
				s1i += x2.x * y2.y + x2.y * y2.x;
			}
			if (e.mode & EPI_DOT_ARG_CONJ) {
				const double2 x2 = to_d2(arg[i * 3 + comp]);
				s1r += x2.x * y2.x + x2.y * y2.y;
				s1i += x2.y * y2.x - x2.x * y2.y;
			}
			if (e.mode & EPI_DOT_U_CONJ) {
				const double2 u2 = to_d2(u[i * 3 + comp]);
				s1r += y2.x * u2.x + y2.y * u2.y;
				s1i += y2.y * u2.x - y2.x * u2.y;
			}
		}
	}
	if (e.mode) {
		const size_t nblk = (size_t)gridDim.x * gridDim.y;
		const size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
		double *out = e.partial + ((size_t)r * nblk + blk) * 4;
		double v0 = block_sum<T>(s0, red);
		double v1 = block_sum<T>(s1r, red);
		double v2 = block_sum<T>(s1i, red);
		if (threadIdx.x == 0) {
			out[0] = v0;
			out[1] = v1;
			out[2] = v2;
		}
	}
}

// sum per-RHS partials (fixed order): out[r*4 + 0..2]
__global__ void reduce_partials_k(const double *partial, size_t nblk, double *out)
{
	__shared__ double red[32];
	const int r = blockIdx.x;
	double s[3] = {0, 0, 0};
	for (size_t b = threadIdx.x; b < nblk; b += blockDim.x)
		for (int j = 0; j < 3; j++) s[j] += partial[((size_t)r * nblk + b) * 4 + j];
	for (int j = 0; j < 3; j++) {
		double v = block_sum<double>(s[j], red);
		if (threadIdx.x == 0) out[r * 4 + j] = v;
	}
}

constexpr int W1_F = 8, W1_D = 4;   // y-lines per K1/K3 tile
constexpr int W2_F = 16, W2_D = 8;  // y-lines per K2a/K2c tile
const size_t SMEM_CAP = 200 * 1024;

template <typename T> struct Tiles;
template <> struct Tiles<float> { static constexpr int W1 = W1_F, W2 = W2_F; };
template <> struct Tiles<double> { static constexpr int W1 = W1_D, W2 = W2_D; };

template <typename T> size_t smem_k1(const adda_gb300_ctx *c)
{
	return 2 * sizeof(typename CxT<T>::type) * (size_t)c->gX * tile_ls(3 * Tiles<T>::W1);
}
template <typename T> size_t smem_k2(const adda_gb300_ctx *c)
{
	return 2 * sizeof(typename CxT<T>::type) * (size_t)c->gZ * tile_ls(Tiles<T>::W2);
}
// choose KB (kz per block) and RG (RHS per block) for K2b so that the tile fits
template <typename T> void k2b_shape(const adda_gb300_ctx *c, int R, int &KB, int &RG, size_t &smem)
{
	const size_t cs = sizeof(typename CxT<T>::type);
	auto sz = [&](int rg, int kb) { return 2 * cs * c->gY * (size_t)tile_ls(rg * 3 * kb); };
	RG = R;
	KB = 4;
	while (KB > 1 && sz(RG, KB) > SMEM_CAP) KB /= 2;
	while (RG > 1 && sz(RG, KB) > SMEM_CAP) RG = (RG + 1) / 2;
	smem = sz(RG, KB);
}

template <typename T, typename V> int set_attrs_v(adda_gb300_ctx *c)
{
	const int W1 = Tiles<T>::W1, W2 = Tiles<T>::W2;
	const size_t s1 = smem_k1<T>(c), s2 = smem_k2<T>(c);
	ADDA_CUDA(cudaFuncSetAttribute(mv_scatter_fftx<T, V, W1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
	ADDA_CUDA(cudaFuncSetAttribute(mv_fftx_gather<T, V, W1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
	ADDA_CUDA(cudaFuncSetAttribute(mv_fftz<T, V, W2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
	ADDA_CUDA(cudaFuncSetAttribute(mv_fftz<T, V, W2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
	ADDA_CUDA(cudaFuncSetAttribute(mv_fft_y_dmul<T, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
	return ADDA_GB300_OK;
}

template <typename T> int set_attrs(adda_gb300_ctx *c)
{
	int KB, RG;
	size_t s2b;
	k2b_shape<T>(c, c->Rmax, KB, RG, s2b);
	const size_t s1 = smem_k1<T>(c), s2 = smem_k2<T>(c);
	if (s1 > 227 * 1024 || s2 > 227 * 1024 || s2b > 227 * 1024) {
		set_error("FFT grid too large for the shared-memory tiles");
		return ADDA_GB300_EINVAL;
	}
	int rc = set_attrs_v<T, typename CxT<T>::type>(c);
	if (rc) return rc;
	if (sizeof(T) == 4) rc = set_attrs_v<T, double2>(c);
	return rc;
}

} // namespace

size_t matvec_partial_blocks(const adda_gb300_ctx *c, bool dbl)
{
	// K3 grid: ceil(bY/W1) x bZ blocks per RHS
	const int w = dbl ? W1_D : W1_F;
	return (size_t)((c->bY + w - 1) / w) * c->bZ;
}

int matvec_setup(adda_gb300_ctx *c)
{
	int rc = set_attrs<float>(c);
	if (rc) return rc;
	rc = set_attrs<double>(c);
	if (rc) return rc;
	return ADDA_GB300_OK;
}

template <typename T, typename V>
int matvec_run(adda_gb300_ctx *c, int R, const V *arg, V *res, int her, const MvEpi &epi, const int *done)
{
	typedef typename CxT<T>::type C;
	const bool dbl = sizeof(T) == 8;
	const int W1 = Tiles<T>::W1, W2 = Tiles<T>::W2;
	MvP<T, V> p;
	p.bX = c->bX; p.bY = c->bY; p.bZ = c->bZ;
	p.gX = c->gX; p.gY = c->gY; p.gZ = c->gZ;
	p.DsY = c->DsY; p.DsZ = c->DsZ;
	p.R = R;
	p.N = c->N;
	p.line_start = c->d_line_start;
	p.xy = c->d_xy;
	p.mat = c->d_mat;
	p.ccs = dbl ? (const C *)c->ccs64 : (const C *)c->ccs32;
	p.nmat = c->nmat;
	p.per_dip = c->per_dip;
	p.arg = arg;
	p.res = res;
	p.Xf = (C *)c->Xf;
	p.Tz = (C *)c->Tz;
	p.CK = dbl ? c->CK64 : c->CK32;
	p.D = dbl ? (const C *)c->D64 : (const C *)c->D32;
	const int pi = dbl ? 0 : 1;
	p.px = c->px[pi]; p.py = c->py[pi]; p.pz = c->pz[pi];
	p.twx = dbl ? (const C *)c->tw64[0] : (const C *)c->tw32[0];
	p.twy = dbl ? (const C *)c->tw64[1] : (const C *)c->tw32[1];
	p.twz = dbl ? (const C *)c->tw64[2] : (const C *)c->tw32[2];
	p.her = her;
	p.done = done;
	p.kx0 = 0;
	cudaStream_t st = c->stream;
	const dim3 blk(256);
	const dim3 g1((c->bY + W1 - 1) / W1, c->bZ, R);
	mv_scatter_fftx<T, V, W1><<<g1, blk, smem_k1<T>(c), st>>>(p);
	ADDA_LAUNCHED();
	int KB, RG;
	size_t s2b;
	k2b_shape<T>(c, R, KB, RG, s2b);
	for (int kx0 = 0; kx0 < c->gX; kx0 += p.CK) {
		p.kx0 = kx0;
		const int ck = std::min(p.CK, c->gX - kx0);
		const dim3 g2((c->bY + W2 - 1) / W2, 3 * ck, R);
		mv_fftz<T, V, W2, false><<<g2, blk, smem_k2<T>(c), st>>>(p);
		ADDA_LAUNCHED();
		const dim3 g2b((c->gZ + KB - 1) / KB, ck, (R + RG - 1) / RG);
		mv_fft_y_dmul<T, V><<<g2b, blk, s2b, st>>>(p, KB, RG);
		ADDA_LAUNCHED();
		mv_fftz<T, V, W2, true><<<g2, blk, smem_k2<T>(c), st>>>(p);
		ADDA_LAUNCHED();
	}
	mv_fftx_gather<T, V, W1><<<g1, blk, smem_k1<T>(c), st>>>(p, epi);
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

template int matvec_run<float, float2>(adda_gb300_ctx *, int, const float2 *, float2 *, int, const MvEpi &,
	const int *);
template int matvec_run<float, double2>(adda_gb300_ctx *, int, const double2 *, double2 *, int, const MvEpi &,
	const int *);
template int matvec_run<double, double2>(adda_gb300_ctx *, int, const double2 *, double2 *, int, const MvEpi &,
	const int *);

int reduce_partials(adda_gb300_ctx *c, int R, const double *partial, size_t nblk, double *out)
{
	reduce_partials_k<<<R, 256, 0, c->stream>>>(partial, nblk, out);
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

} // namespace adda
