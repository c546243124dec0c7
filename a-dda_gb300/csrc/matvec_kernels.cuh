// matvec_kernels.cuh - the kernels of the FFT-accelerated DDA matvec y = x + S.D.S.x (MatVec, src/matvec.c:128).
//
// Data flow for R right-hand sides sharing one interaction matrix D (all in HBM unless noted):
//   K1 mv_scatter_fftx : per (rhs, z, block of W y-lines): gather S.x of the dipoles of those x-lines straight from
//                        the dipole vector (no zeroed expanded grid, the reference's Xmatrix fill + Arith1), pad to
//                        gridX in shared memory, forward FFT along x  ->  Xf[r][kx][comp][z][y]
//   then per chunk of CK x-slabs (chunk buffer Tz sized to stay in L2):
//   K2a mv_fftz        : forward FFT along z of each y-line block (z>=boxZ zero: only z<gZ/2 is read)
//   K2b mv_fft_y_dmul  : per (kx, kz block, RHS group): forward FFT along y, 6-component symmetric D~ x X~ product
//                        (D read once per grid point and reused by every RHS of the block), inverse FFT along y;
//       mv_fft_y_reg   : the same in register form (FP32, power-of-two gY <= 512): one lane group per column, lines
//                        straight from Tz into registers, in-register two-step FFT, no block barrier
//   K2c mv_fftz (inv)  : inverse FFT along z, keep z<boxZ  ->  Xf
//   K3 mv_fftx_gather  : inverse FFT along x, y = x + S.X for the dipoles of the lines, optional Krylov reductions
//                        (|y|^2, x.y, y.u*, x.y*) as deterministic per-block partial sums.
// Every kernel skips the right-hand sides the solver has finished (rhs_done).
// A particle near a substrate adds, per chunk, K2a in its third mode (the same slab transformed along z with the
// inverse sign into TzR, so that the product sums heights) and K2b in its surface forms (mv_fft_y_surf, or
// mv_fft_y_reg<..., true>): D~.X~ + R~.X'~ before the inverse y transform (matvec.c:249-303).
// The reference's explicit transposes (TransposeYZ), slice zeroing and copies (Arith2/Arith4) do not exist here:
// every line is read and written along the contiguous axis of its buffer (y), whichever axis it transforms.
// Every kernel is instantiated with a compile-time FFT length NS for the power-of-two grids (all index arithmetic
// folds to shifts, passes unroll) and with NS = 0 (runtime plan) for the other fftFit sizes. With FP32 arithmetic and
// a power-of-two length the lines are transformed in registers (lf_fft: 8-16 threads per line, consecutive threads
// on consecutive lines, one exchange through shared memory, the zero half of every padded line skipped); blocks then
// have lines x threads-per-line threads, otherwise 256 threads and ping-pong Stockham passes over two tiles.
#pragma once

#include "ctx.cuh"

#include <algorithm>

namespace adda {
namespace mv {

// T = arithmetic of the FFTs, D and the expanded grid (float or double); V = complex type of the dipole vectors the
// caller passes (float2, double2 or double-float dd2). With T=float and V=double2 or dd2 (the MIXED solvers) the
// inputs are rounded on the fly and y = x + S.X is accumulated in the vector's precision, so the identity part of A
// keeps that precision.
// Everything but the dipole vectors: the y/z stage (K2a, K2b, K2c) never touches them, so its kernels are compiled
// once per arithmetic type T.
template <typename T> struct MvGeom {
	typedef typename CxT<T>::type C;
	int bX, bY, bZ, gX, gY, gZ, DsY, DsZ;
	int R;
	size_t N;
	const uint32_t *line_start;
	const uint32_t *xy;
	const uint8_t *mat;
	const C *ccs;   // per-RHS cc_sqrt: [R][nmat][3] or [R][N][3]
	int nmat, per_dip;
	C *Xf;
	C *Tz;
	int CK, kx0;
	const C *D;
	FftPlan px, py, pz;
	const C *twx, *twy, *twz;
	int her;
	int KB, RG;      // K2b: kz per block, RHS per block (KB*RG <= Tiles<T>::PAIRS)
	const int *done; // per-RHS done flags (may be null): every kernel returns at once when all are set
	// particle near a substrate: the slab transformed along z with the opposite sign (height sums) and the
	// reflected interaction matrix R~, layout [gX][gZ][RsY][6] (fft.c:196-201)
	C *TzR;
	const C *Rm;
	int RsY;
	int rpp;           // RHS per particle: RHS r uses lattice slot r / rpp (a group context, adda_gb300_create_group)
	size_t lat_stride; // dipoles per lattice slot
};

template <typename T, typename V> struct MvP : MvGeom<T> {
	const V *arg;
	V *res;
};

template <typename To, typename From> __device__ __forceinline__ To cvt(From a) { return from_d2<To>(to_d2(a)); }
// double-float vectors: round to float on load (K1) and widen the float S.X exactly (K3), all on the FP32 pipes
template <> __device__ __forceinline__ float2 cvt<float2, dd2>(dd2 a) { return p_add(a.h, a.l); }
template <> __device__ __forceinline__ dd2 cvt<dd2, float2>(float2 a) { return dd2{a, make_float2(0.f, 0.f)}; }

// Xf (the x-transformed half grid, 201 MB at 256^3 and 2 RHS) is written once and read once per matvec: its loads
// and stores by the column kernels are marked streaming (evict first), so that the L2 keeps the chunk buffer Tz and
// the D rows instead (matvec 0.691 -> 0.672 ms at 256^3, bit-identical results)
#define XF_LD(ptr) __ldcs(ptr)
#define XF_ST(ptr, val) __stcs((ptr), (val))
template <typename P> __device__ __forceinline__ bool all_done(const P &p)
{
	if (!p.done) return false;
	for (int r = 0; r < p.R; r++)
		if (!p.done[r]) return false;
	return true;
}
// a right-hand side the solver has finished (converged, broken down or stopped): the matvec skips its blocks, since
// every vector kernel and scalar kernel of the solver leaves a finished RHS alone and nothing reads its products
template <typename P> __device__ __forceinline__ bool rhs_done(const P &p, int r) { return p.done && p.done[r]; }

template <typename C> __device__ __forceinline__ C ccs_of(const C *ccs, int per_dip, int nmat, size_t N, int r,
	size_t i, uint8_t m, int comp)
{
	return per_dip ? ccs[((size_t)r * N + i) * 3 + comp] : ccs[((size_t)r * nmat + m) * 3 + comp];
}

// tile widths: W1 y-lines per K1/K3 block, W2 y-lines per K2a/K2c block, PAIRS (RHS, kz) pairs per K2b block
template <typename T> struct Tiles;
template <> struct Tiles<float> { static constexpr int W1 = 8, W2 = 16, PAIRS = 8; };
template <> struct Tiles<double> { static constexpr int W1 = 4, W2 = 8, PAIRS = 4; };

// K1: scatter S.x of W consecutive x-lines (one z) into shared memory and FFT along x. Tile: gX x (3*W) lines.
template <typename T, typename V, int W, int NS>
__global__ void __launch_bounds__(col_threads<T, NS, 3 * W>(), (col_minblocks<T, NS, 3 * W>()))
	mv_scatter_fftx(MvP<T, V> p)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (rhs_done(p, blockIdx.z)) return; // blockIdx.z = RHS
	constexpr int NL = 3 * W, LS = tile_ls(3 * W), NT = col_threads<T, NS, 3 * W>();
	constexpr bool RC = reg_cols<T, NS>();
	const int n = NS ? NS : p.gX;
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)n * LS; // second tile of the Stockham form only
	const int r = blockIdx.z, z = blockIdx.y, y0 = blockIdx.x * W;
	// the lattice of RHS r's particle (a single-lattice context has one)
	const size_t lq = (size_t)(r / p.rpp);
	const uint32_t *lstart = p.line_start + lq * ((size_t)p.bZ * p.bY + 1), *lxy = p.xy + lq * p.lat_stride;
	const uint8_t *lmat = p.mat + lq * p.lat_stride;
	const int wy = min(W, p.bY - y0);
	// the column form reads elements x < gX/2 only (gX >= 2 bX for the power-of-two lengths it is built for)
	for (int t = threadIdx.x; t < (RC ? n / 2 : n) * LS; t += NT) a[t] = cx<C>(0, 0);
	__syncthreads();
	const size_t line = (size_t)z * p.bY + y0;
	const uint32_t i0 = lstart[line], i1 = lstart[line + wy];
	const V *arg = p.arg + (size_t)r * p.N * 3;
#pragma unroll 2
	for (uint32_t i = i0 + threadIdx.x; i < i1; i += NT) {
		const uint32_t q = lxy[i];
		const int x = q & 0xffff, y = q >> 16;
		const uint8_t m = lmat[i];
#pragma unroll
		for (int comp = 0; comp < 3; comp++) {
			C v = cvt<C>(arg[(size_t)i * 3 + comp]);
			if (p.her) v = cconj(v);
			v = cmul(ccs_of(p.ccs, p.per_dip, p.nmat, p.N, r, i, m, comp), v);
			a[x * LS + comp * W + (y - y0)] = v;
		}
	}
	__syncthreads();
	const size_t plane = (size_t)p.bZ * p.bY;
	C *xf = p.Xf + (size_t)r * p.gX * 3 * plane + (size_t)z * p.bY + y0;
	if constexpr (RC) {
		// line-fastest transform of the tile's lines l = comp*W + yy; each thread stores its elements kx of line l
		// straight to Xf (consecutive threads = consecutive y)
		constexpr int TL = RegShape<NS>::T, E = RegShape<NS>::E;
		const int l = threadIdx.x % NL, j1 = threadIdx.x / NL, comp = l / W, yy = l % W;
		C v[E];
#pragma unroll
		for (int j = 0; j < E / 2; j++) v[j] = a[(j1 + TL * j) * LS + l];
		__syncthreads(); // the exchange buffer of lf_fft overwrites the tile
		lf_fft<C, NS, NL, false, true>(v, a, l, j1, p.twx);
		if (yy < wy) {
			C *dst = xf + (size_t)comp * plane + yy;
#pragma unroll
			for (int i = 0; i < E / TL; i++)
#pragma unroll
				for (int k1 = 0; k1 < TL; k1++) XF_ST(dst + (size_t)(j1 + i * TL + E * k1) * 3 * plane, v[i * TL + k1]);
		}
	}
	else {
		const C *o = tile_fft<C, NS, NL, LS, false>(a, b, p.px, p.twx);
		for (int t = threadIdx.x; t < n * NL; t += NT) {
			const int yy = t % W, rest = t / W;
			const int comp = rest % 3, kx = rest / 3;
			if (yy < wy) xf[((size_t)kx * 3 + comp) * plane + yy] = o[kx * LS + comp * W + yy];
		}
	}
}

// K2a/K2c: FFT along z of W consecutive y-lines of one (rhs, kx, comp). MODE 0 (forward) reads Xf (z<bZ, zero
// padded) and writes Tz (all kz); MODE 1 (inverse) reads Tz and writes z<bZ back to Xf; MODE 2 (surface) reads Xf
// like MODE 0 but transforms with the inverse sign into TzR, so that the product with R~ sums heights instead of
// differences (planZRf, fft.c:396-403, matvec.c:249).
// FP32 with a power-of-two length (the column form): thread (l, j1) = (threadIdx % W, threadIdx / W) holds elements
// z = j1 + T*j of y-line l in registers, read and written straight from and to HBM/L2 (consecutive threads =
// consecutive y: coalesced rows, no staging tile), and the two-step FFT exchanges its intermediate through shared
// memory laid out [k2][j1][l] (one block barrier; both phases conflict-free, a pad of W elements per k2 row group
// for W = 8). The forward transforms read z < gZ/2 only and start with dft_half_in; the inverse keeps z < gZ/2.
// Otherwise a staged tile and Stockham passes.
template <typename T, int W, int MODE, int NS>
__global__ void __launch_bounds__(col_threads<T, NS, W>(), (col_minblocks<T, NS, W>())) mv_fftz(MvGeom<T> p)
{
	constexpr bool INV = MODE == 1, SGN = MODE != 0;
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (rhs_done(p, blockIdx.z)) return; // blockIdx.z = RHS
	constexpr int LS = tile_ls(W), NT = col_threads<T, NS, W>();
	constexpr bool RC = reg_cols<T, NS>();
	const int n = NS ? NS : p.gZ;
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)n * LS;
	const int r = blockIdx.z;
	const int kxl = blockIdx.y / 3, comp = blockIdx.y % 3;
	const int kx = p.kx0 + kxl;
	const int y0 = blockIdx.x * W;
	const int wy = min(W, p.bY - y0);
	const size_t plane = (size_t)p.bZ * p.bY;
	C *xf = p.Xf + (((size_t)r * p.gX + kx) * 3 + comp) * plane + y0;
	C *tz = (MODE == 2 ? p.TzR : p.Tz) + (((size_t)r * p.CK + kxl) * 3 + comp) * (size_t)n * p.bY + y0;
	if constexpr (RC) {
		constexpr int TL = RegShape<NS>::T, E = RegShape<NS>::E;
		const int l = threadIdx.x % W, j1 = threadIdx.x / W;
		const bool yok = l < wy;
		const size_t ys = (size_t)p.bY;
		C v[E];
		if constexpr (INV) {
#pragma unroll
			for (int j = 0; j < E; j++) v[j] = yok ? __ldg(tz + (size_t)(j1 + TL * j) * ys + l) : cx<C>(0, 0);
		}
		else {
#pragma unroll
			for (int j = 0; j < E / 2; j++) {
				const int z = j1 + TL * j;
				v[j] = (yok && z < p.bZ) ? XF_LD(xf + (size_t)z * ys + l) : cx<C>(0, 0);
			}
		}
		lf_fft<C, NS, W, SGN, !INV>(v, a, l, j1, p.twz);
		// v[i*TL + k1] = element (j1 + i*TL) + E*k1 of the transformed line
		if (yok) {
#pragma unroll
			for (int i = 0; i < E / TL; i++) {
				if constexpr (INV) {
#pragma unroll
					for (int k1 = 0; k1 < TL / 2; k1++) {
						const int z = j1 + i * TL + E * k1;
						if (z < p.bZ) XF_ST(xf + (size_t)z * ys + l, v[i * TL + k1]);
					}
				}
				else {
#pragma unroll
					for (int k1 = 0; k1 < TL; k1++) tz[(size_t)(j1 + i * TL + E * k1) * ys + l] = v[i * TL + k1];
				}
			}
		}
		return;
	}
	else {
		// NT is a multiple of W: each thread keeps one y-line and walks z with a constant stride
		constexpr int ZS = NT / W;
		const int yy = threadIdx.x % W, z0 = threadIdx.x / W;
		const bool yok = yy < wy;
		{
			const C *src = (INV ? tz : xf) + (size_t)z0 * p.bY + yy;
			const C *base = INV ? tz : xf;
			const size_t step = (size_t)ZS * p.bY;
#pragma unroll 4
			for (int z = z0; z < n; z += ZS, src += step) {
				const bool ok = yok && (INV || z < p.bZ);
				cp_async_elem(a + z * LS + yy, ok ? src : base, ok);
			}
		}
		cp_async_commit();
		cp_async_wait<0>();
		__syncthreads();
		C *o = tile_fft<C, NS, W, LS, SGN>(a, b, p.pz, p.twz);
		const int zmax = INV ? p.bZ : n;
		if (yok) {
			C *dst = (INV ? xf : tz) + (size_t)z0 * p.bY + yy;
			const size_t step = (size_t)ZS * p.bY;
#pragma unroll 4
			for (int z = z0; z < zmax; z += ZS, dst += step) *dst = o[z * LS + yy];
		}
	}
}

// K2b: per (kx, KB kz, RG RHS) with KB*RG <= P pairs: y-FFT of the 3 components, D product (matvec.c:271-305 incl. the
// reduced-FFT signs), inverse y-FFT. Line l = pair*3 + comp, pair = kk*RG + rr. Warp w loads/stores lines w, w+8, w+16
// with its 32 lanes along y (coalesced rows of Tz, odd tile stride: conflict-free).
template <typename T, int NS, int P> __global__ void __launch_bounds__(256) mv_fft_y_dmul(MvGeom<T> p)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	constexpr int NL = 3 * P, LS = tile_ls(NL);
	const int n = NS ? NS : p.gY;
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)n * LS;
	const int KB = p.KB, RG = p.RG;
	const int rg0 = blockIdx.z * RG;
	{
		bool live = false; // any of the block's RHS still running
		for (int rr = rg0; rr < min(rg0 + RG, p.R); rr++) live = live || !rhs_done(p, rr);
		if (!live) return;
	}
	const int kxl = blockIdx.y, kx = p.kx0 + kxl;
	const int kz0 = blockIdx.x * KB;
	const size_t lz = (size_t)p.gZ * p.bY; // one (rhs, kx, comp) block of Tz
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	for (int l = warp; l < NL; l += 8) {
		const int pair = l / 3, comp = l - 3 * pair;
		const int kk = pair / RG, rr = pair - kk * RG;
		const int kz = kz0 + kk;
		const bool ok = kk < KB && rg0 + rr < p.R && kz < p.gZ;
		const C *src = p.Tz + (((size_t)(rg0 + rr) * p.CK + kxl) * 3 + comp) * lz + (size_t)kz * p.bY;
#pragma unroll 4
		for (int y = lane; y < n; y += 32) a[y * LS + l] = (ok && y < p.bY) ? src[y] : cx<C>(0, 0);
	}
	__syncthreads();
	C *o = tile_fft<C, NS, NL, LS, false>(a, b, p.py, p.twy);
	C *s = (o == a) ? b : a;
	for (int t = threadIdx.x; t < KB * n; t += 256) {
		const int ky = t % n, kk = t / n;
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
		const int rgn = min(RG, p.R - rg0);
		for (int rr = 0; rr < rgn; rr++) {
			const int l0 = (kk * RG + rr) * 3;
			C *row = o + ky * LS + l0;
			const C v0 = row[0], v1 = row[1], v2 = row[2];
			row[0] = cfma(m0, v0, cfma(m1, v1, cmul(m2, v2)));
			row[1] = cfma(m1, v0, cfma(m3, v1, cmul(m4, v2)));
			row[2] = cfma(m2, v0, cfma(m4, v1, cmul(m5, v2)));
		}
	}
	__syncthreads();
	C *o2 = tile_fft<C, NS, NL, LS, true>(o, s, p.py, p.twy);
	for (int l = warp; l < NL; l += 8) {
		const int pair = l / 3, comp = l - 3 * pair;
		const int kk = pair / RG, rr = pair - kk * RG;
		const int kz = kz0 + kk;
		if (!(kk < KB && rg0 + rr < p.R && kz < p.gZ)) continue;
		C *dst = p.Tz + (((size_t)(rg0 + rr) * p.CK + kxl) * 3 + comp) * lz + (size_t)kz * p.bY;
		for (int y = lane; y < p.bY; y += 32) dst[y] = o2[y * LS + l];
	}
}

// K2b for a particle near a substrate (matvec.c:255-305): per (kx, KB kz, RG RHS) with KB*RG <= P/2, six lines
// per pair: the 3 components of Tz and of TzR. All are transformed along y; then yv = D~.xv + R~.xvR with D's
// reduced-FFT signs and R's (reduced in y only: xy and yz change sign for ky > gY/2) and R's product
// M21 = M12, M31 = -M13, M32 = -M23 (cReflMatrVec, cmplx.h:391-401); the result goes back through the inverse y
// transform into Tz. Line l = pair*6 + c6, c6 < 3 from Tz, c6 >= 3 from TzR.
template <typename T, int NS, int P> __global__ void __launch_bounds__(256) mv_fft_y_surf(MvGeom<T> p)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	constexpr int NL = 3 * P, LS = tile_ls(NL);
	const int n = NS ? NS : p.gY;
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)n * LS;
	const int KB = p.KB, RG = p.RG;
	const int rg0 = blockIdx.z * RG;
	{
		bool live = false; // any of the block's RHS still running
		for (int rr = rg0; rr < min(rg0 + RG, p.R); rr++) live = live || !rhs_done(p, rr);
		if (!live) return;
	}
	const int kxl = blockIdx.y, kx = p.kx0 + kxl;
	const int kz0 = blockIdx.x * KB;
	const size_t lz = (size_t)p.gZ * p.bY;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	for (int l = warp; l < NL; l += 8) {
		const int pair = l / 6, c6 = l - 6 * pair, comp = c6 % 3;
		const int kk = pair / RG, rr = pair - kk * RG;
		const int kz = kz0 + kk;
		const bool ok = kk < KB && rg0 + rr < p.R && kz < p.gZ;
		const C *src = (c6 < 3 ? p.Tz : p.TzR) + (((size_t)(rg0 + rr) * p.CK + kxl) * 3 + comp) * lz +
			(size_t)kz * p.bY;
#pragma unroll 4
		for (int y = lane; y < n; y += 32) a[y * LS + l] = (ok && y < p.bY) ? src[y] : cx<C>(0, 0);
	}
	__syncthreads();
	C *o = tile_fft<C, NS, NL, LS, false>(a, b, p.py, p.twy);
	C *s = (o == a) ? b : a;
	for (int t = threadIdx.x; t < KB * n; t += 256) {
		const int ky = t % n, kk = t / n;
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
		const bool qy = ky >= p.RsY;
		const C *g = p.Rm + (((size_t)kx * p.gZ + kz) * p.RsY + (qy ? p.gY - ky : ky)) * 6;
		C q0 = g[0], q1 = g[1], q2 = g[2], q3 = g[3], q4 = g[4], q5 = g[5];
		if (qy) {
			q1 = cneg(q1);
			q4 = cneg(q4);
		}
		const int rgn = min(RG, p.R - rg0);
		for (int rr = 0; rr < rgn; rr++) {
			C *row = o + ky * LS + (kk * RG + rr) * 6;
			const C v0 = row[0], v1 = row[1], v2 = row[2], u0 = row[3], u1 = row[4], u2 = row[5];
			const C w0 = cfma(q0, u0, cfma(q1, u1, cmul(q2, u2)));
			const C w1 = cfma(q1, u0, cfma(q3, u1, cmul(q4, u2)));
			const C w2 = cfma(q5, u2, cneg(cfma(q2, u0, cmul(q4, u1))));
			row[0] = cadd(w0, cfma(m0, v0, cfma(m1, v1, cmul(m2, v2))));
			row[1] = cadd(w1, cfma(m1, v0, cfma(m3, v1, cmul(m4, v2))));
			row[2] = cadd(w2, cfma(m2, v0, cfma(m4, v1, cmul(m5, v2))));
		}
	}
	__syncthreads();
	C *o2 = tile_fft<C, NS, NL, LS, true>(o, s, p.py, p.twy);
	for (int l = warp; l < NL; l += 8) {
		const int pair = l / 6, c6 = l - 6 * pair;
		const int kk = pair / RG, rr = pair - kk * RG;
		const int kz = kz0 + kk;
		if (c6 >= 3 || !(kk < KB && rg0 + rr < p.R && kz < p.gZ)) continue;
		C *dst = p.Tz + (((size_t)(rg0 + rr) * p.CK + kxl) * 3 + c6) * lz + (size_t)kz * p.bY;
		for (int y = lane; y < p.bY; y += 32) dst[y] = o2[y * LS + l];
	}
}

// K2b, register form for FP32 and power-of-two gY <= 512: one group of T lanes per (kx, kz, rhs) column; each
// component line goes from Tz straight into registers (lane j1 holds y = j1 + T*j: half-warp rows of 128 B) and is
// transformed by reg_fft (one transpose through a slot of the group's shared memory, no block barrier). The spectra
// of components 0 and 1 are parked in their slots (lane-interleaved: conflict-free) while component 2 stays in
// registers; the 6-component D product at every ky the lane holds (matvec.c:271-305 incl. the reduced-FFT signs)
// writes back to the same places, then each component is transformed back and stored for y < bY. Groups of one block
// cover consecutive (kz, rhs) units with the RHS fastest, so the D rows a block reads are shared through L1.
// SURF (particle near a substrate): after the D product the three TzR lines of the column follow one at a time
// through a fourth slot (the next one loading into the free third slot meanwhile); each spectrum u_c adds column c of
// the reflected product R~.u (M21 = M12, M31 = -M13, M32 = -M23, cReflMatrVec cmplx.h:391-401; R reduced in y only)
// to the three result components before the inverse transforms.
template <int NS, int NT, bool SURF = false>
__global__ void __launch_bounds__(NT, NS >= 512 ? (NT >= 256 ? 1 : 256 / NT) : (SURF ? 3 : 4) * 128 / NT)
	mv_fft_y_reg(MvGeom<float> p)
{
	typedef float2 C;
	constexpr int T = RegShape<NS>::T, E = RegShape<NS>::E, BUF = RegShape<NS>::BUF, G = NT / T;
	constexpr int NSLOT = SURF ? 4 : 3;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (all_done(p)) return;
	const int g = threadIdx.x / T, j1 = threadIdx.x % T;
	const int unit = blockIdx.x * G + g;
	const int r = unit % p.R, kz = unit / p.R;
	if (kz >= p.gZ || rhs_done(p, r)) return; // whole groups leave together
	const unsigned gmask = ((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1));
	const int kxl = blockIdx.y, kx = p.kx0 + kxl;
	C *slot = reinterpret_cast<C *>(smem_raw) + (size_t)g * NSLOT * BUF; // slots c*BUF, c = 0..NSLOT-1
	constexpr int DY = NS / 2 + 1; // rows of D (and R) along y: gY/2 + 1, gY = NS
	const size_t lz = (size_t)p.gZ * p.bY;
	C *col = p.Tz + (((size_t)r * p.CK + kxl) * 3) * lz + (size_t)kz * p.bY;
	// the column's D row (and R row) start moving into L2 now, so that the product after the forward transforms
	// finds them there; one lane of the first RHS's group asks (rows of 6 complex per ky: multiples of 48 bytes)
	if (j1 == 0 && r == 0) {
		prefetch_l2_bulk(p.D + ((size_t)kx * p.DsZ + (kz >= p.DsZ ? p.gZ - kz : kz)) * DY * 6,
			(unsigned)(DY * 6 * sizeof(C)));
		if constexpr (SURF) prefetch_l2_bulk(p.Rm + ((size_t)kx * p.gZ + kz) * DY * 6, (unsigned)(DY * 6 * sizeof(C)));
	}
	// the three component lines go to their slots asynchronously (lane j1 writes and later reads only its own
	// elements, at j*T + j1), one commit group each, so components 1 and 2 arrive during component 0's transform;
	// y < bY <= gY/2, so only the first E/2 elements of a lane can be non-zero (the transforms start with
	// dft_half_in) and only those are stored after the inverse ones
#pragma unroll
	for (int c = 0; c < 3; c++) {
#pragma unroll
		for (int j = 0; j < E / 2; j++) {
			const int y = j1 + T * j;
			if (y < p.bY) cp_async_elem(slot + c * BUF + j * T + j1, col + c * lz + y, true);
		}
		cp_async_commit();
	}
	const C *colR = SURF ? p.TzR + (((size_t)r * p.CK + kxl) * 3) * lz + (size_t)kz * p.bY : nullptr;
	if constexpr (SURF) { // u_0 into slot 3
#pragma unroll
		for (int j = 0; j < E / 2; j++) {
			const int y = j1 + T * j;
			if (y < p.bY) cp_async_elem(slot + 3 * BUF + j * T + j1, colR + y, true);
		}
		cp_async_commit();
	}
	C v[E];
#pragma unroll
	for (int c = 0; c < 3; c++) {
		if (c == 0) cp_async_wait<SURF ? 3 : 2>();
		else if (c == 1) cp_async_wait<SURF ? 2 : 1>();
		else cp_async_wait<SURF ? 1 : 0>();
#pragma unroll
		for (int j = 0; j < E / 2; j++) {
			const int y = j1 + T * j;
			v[j] = (y < p.bY) ? slot[c * BUF + j * T + j1] : make_float2(0.f, 0.f);
		}
		reg_fft<C, NS, false, true>(v, slot + c * BUF, j1, gmask, p.twy + NS);
		reg_natural<C, NS>(v);
		if (c < 2) {
			__syncwarp(gmask);
#pragma unroll
			for (int j = 0; j < E; j++) slot[c * BUF + j * T + j1] = v[j];
		}
	}
	const bool rz = kz >= p.DsZ;
	const int zz = rz ? p.gZ - kz : kz;
	const float4 *drow = reinterpret_cast<const float4 *>(p.D + ((size_t)kx * p.DsZ + zz) * DY * 6);
#pragma unroll
	for (int j = 0; j < E; j++) {
		const int ky = j1 + T * j;
		const bool ry = ky >= DY;
		const int yy = ry ? NS - ky : ky;
		const float4 *f = drow + (size_t)yy * 3;
		const float4 d0 = __ldg(f), d1 = __ldg(f + 1), d2 = __ldg(f + 2);
		C m0 = make_float2(d0.x, d0.y), m1 = make_float2(d0.z, d0.w), m2 = make_float2(d1.x, d1.y);
		C m3 = make_float2(d1.z, d1.w), m4 = make_float2(d2.x, d2.y), m5 = make_float2(d2.z, d2.w);
		if (ry) m1 = cneg(m1);
		if (ry != rz) m4 = cneg(m4);
		if (rz) m2 = cneg(m2);
		const C v0 = slot[j * T + j1], v1 = slot[BUF + j * T + j1], v2 = v[j];
		slot[j * T + j1] = cfma(m0, v0, cfma(m1, v1, cmul(m2, v2)));
		slot[BUF + j * T + j1] = cfma(m1, v0, cfma(m3, v1, cmul(m4, v2)));
		v[j] = cfma(m2, v0, cfma(m4, v1, cmul(m5, v2)));
	}
	if constexpr (SURF) {
		const float4 *rrow = reinterpret_cast<const float4 *>(p.Rm + ((size_t)kx * p.gZ + kz) * DY * 6);
#pragma unroll 1
		for (int c = 0; c < 3; c++) {
			C *ub = slot + (c == 1 ? 2 : 3) * BUF; // u_0 and u_2 in slot 3, u_1 in slot 2 (free after component 2)
			if (c < 2) {
				// the next line into the other slot: slot 2 is free, slot 3 once u_0's transform is done
				__syncwarp(gmask);
				C *nb = slot + (c == 0 ? 2 : 3) * BUF;
#pragma unroll
				for (int j = 0; j < E / 2; j++) {
					const int y = j1 + T * j;
					if (y < p.bY) cp_async_elem(nb + j * T + j1, colR + (size_t)(c + 1) * lz + y, true);
				}
				cp_async_commit();
				cp_async_wait<1>();
			}
			else cp_async_wait<0>();
			C u[E];
#pragma unroll
			for (int j = 0; j < E / 2; j++) {
				const int y = j1 + T * j;
				u[j] = (y < p.bY) ? ub[j * T + j1] : make_float2(0.f, 0.f);
			}
			reg_fft<C, NS, false, true>(u, ub, j1, gmask, p.twy + NS);
			reg_natural<C, NS>(u);
#pragma unroll
			for (int j = 0; j < E; j++) {
				const int ky = j1 + T * j;
				const bool qy = ky >= DY;
				const float4 *f = rrow + (size_t)(qy ? NS - ky : ky) * 3;
				const float4 d0 = __ldg(f), d1 = __ldg(f + 1), d2 = __ldg(f + 2);
				C a0, a1, a2; // column c of R~ with the reduced-y signs of xy and yz
				if (c == 0) {
					a0 = make_float2(d0.x, d0.y);
					a1 = make_float2(d0.z, d0.w);
					a2 = make_float2(-d1.x, -d1.y);
					if (qy) a1 = cneg(a1);
				}
				else if (c == 1) {
					a0 = make_float2(d0.z, d0.w);
					a1 = make_float2(d1.z, d1.w);
					a2 = make_float2(-d2.x, -d2.y);
					if (qy) {
						a0 = cneg(a0);
						a2 = cneg(a2);
					}
				}
				else {
					a0 = make_float2(d1.x, d1.y);
					a1 = make_float2(d2.x, d2.y);
					a2 = make_float2(d2.z, d2.w);
					if (qy) a1 = cneg(a1);
				}
				slot[j * T + j1] = cfma(a0, u[j], slot[j * T + j1]);
				slot[BUF + j * T + j1] = cfma(a1, u[j], slot[BUF + j * T + j1]);
				v[j] = cfma(a2, u[j], v[j]);
			}
		}
		__syncwarp(gmask);
	}
#pragma unroll 1
	for (int c = 2; c >= 0; c--) {
		if (c < 2) {
#pragma unroll
			for (int j = 0; j < E; j++) v[j] = slot[c * BUF + j * T + j1];
		}
		reg_fft<C, NS, true>(v, slot + c * BUF, j1, gmask, p.twy + NS);
		reg_natural<C, NS>(v);
#pragma unroll
		for (int j = 0; j < E / 2; j++) {
			const int y = j1 + T * j;
			if (y < p.bY) col[c * lz + y] = v[j];
		}
	}
}

__device__ __forceinline__ double block_sum(double v, double *sh)
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
template <typename T, typename V, int W, int NS>
__global__ void __launch_bounds__(col_threads<T, NS, 3 * W>(), (col_minblocks<T, NS, 3 * W>()))
	mv_fftx_gather(MvP<T, V> p, MvEpi e)
{
	typedef typename CxT<T>::type C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ double red[32];
	if (rhs_done(p, blockIdx.z)) return; // blockIdx.z = RHS
	constexpr int NL = 3 * W, LS = tile_ls(3 * W), NT = col_threads<T, NS, 3 * W>();
	constexpr bool RC = reg_cols<T, NS>();
	const int n = NS ? NS : p.gX;
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)n * LS;
	const int r = blockIdx.z, z = blockIdx.y, y0 = blockIdx.x * W;
	// the lattice of RHS r's particle (a single-lattice context has one)
	const size_t lq = (size_t)(r / p.rpp);
	const uint32_t *lstart = p.line_start + lq * ((size_t)p.bZ * p.bY + 1), *lxy = p.xy + lq * p.lat_stride;
	const uint8_t *lmat = p.mat + lq * p.lat_stride;
	const int wy = min(W, p.bY - y0);
	const size_t plane = (size_t)p.bZ * p.bY;
	const C *xf = p.Xf + (size_t)r * p.gX * 3 * plane + (size_t)z * p.bY + y0;
	C *o = a;
	if constexpr (RC) {
		// line-fastest transform of lines l = comp*W + yy read straight from Xf (consecutive threads = consecutive
		// y); the result rows x < bX <= gX/2, the only ones gathered, go to the tile in natural order
		constexpr int TL = RegShape<NS>::T, E = RegShape<NS>::E;
		const int l = threadIdx.x % NL, j1 = threadIdx.x / NL, comp = l / W, yy = l % W;
		const bool ok = yy < wy;
		const C *src = xf + (size_t)comp * plane + yy;
		C v[E];
#pragma unroll
		for (int j = 0; j < E; j++) v[j] = ok ? XF_LD(src + (size_t)(j1 + TL * j) * 3 * plane) : cx<C>(0, 0);
		lf_fft<C, NS, NL, true, false>(v, a, l, j1, p.twx);
		__syncthreads(); // every exchange read is done before the result rows overwrite the buffer
#pragma unroll
		for (int i = 0; i < E / TL; i++)
#pragma unroll
			for (int k1 = 0; k1 < TL / 2; k1++) a[(j1 + i * TL + E * k1) * LS + l] = v[i * TL + k1];
		__syncthreads();
	}
	else {
#pragma unroll 4
		for (int t = threadIdx.x; t < n * NL; t += NT) {
			const int yy = t % W, rest = t / W;
			const int comp = rest % 3, kx = rest / 3;
			const bool ok = yy < wy;
			cp_async_elem(a + kx * LS + comp * W + yy, ok ? xf + ((size_t)kx * 3 + comp) * plane + yy : xf, ok);
		}
		cp_async_commit();
		cp_async_wait<0>();
		__syncthreads();
		o = tile_fft<C, NS, NL, LS, true>(a, b, p.px, p.twx);
	}
	const size_t line = (size_t)z * p.bY + y0;
	const uint32_t i0 = lstart[line], i1 = lstart[line + wy];
	const V *arg = p.arg + (size_t)r * p.N * 3;
	V *res = p.res + (size_t)r * p.N * 3;
	const V *u = e.u ? reinterpret_cast<const V *>(e.u) + (size_t)r * p.N * 3 : nullptr;
	typename AccOf<V>::T s0{}, s1r{}, s1i{};
	for (uint32_t i = i0 + threadIdx.x; i < i1; i += NT) {
		const uint32_t q = lxy[i];
		const int x = q & 0xffff, y = q >> 16;
		const uint8_t m = lmat[i];
#pragma unroll
		for (int comp = 0; comp < 3; comp++) {
			const size_t j = (size_t)i * 3 + comp;
			const V x0 = arg[j];
			const V xv = p.her ? cconj(x0) : x0;
			const C sx = cmul(ccs_of(p.ccs, p.per_dip, p.nmat, p.N, r, i, m, comp), o[x * LS + comp * W + (y - y0)]);
			V yv = cadd(xv, cvt<V>(sx));
			if (p.her) yv = cconj(yv);
			res[j] = yv;
			if (e.mode) {
				if (e.mode & EPI_NORM) acc_abs2(s0, yv);
				if (e.mode & EPI_DOT_ARG) acc_cmul(s1r, s1i, x0, yv);      // x.y
				if (e.mode & EPI_DOT_ARG_CONJ) acc_cmulc(s1r, s1i, x0, yv); // x.y*
				if (e.mode & EPI_DOT_U_CONJ) acc_cmulc(s1r, s1i, yv, u[j]);  // y.u*
			}
		}
	}
	if (e.mode) {
		const size_t nblk = (size_t)gridDim.x * gridDim.y;
		const size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
		double *out = e.partial + ((size_t)r * nblk + blk) * 4;
		double v0 = block_sum(acc_val(s0), red);
		double v1 = block_sum(acc_val(s1r), red);
		double v2 = block_sum(acc_val(s1i), red);
		if (threadIdx.x == 0) {
			out[0] = v0;
			out[1] = v1;
			out[2] = v2;
		}
	}
}

// ---------------------------------------------------------------------------------------------------------------
// host side

// compile-time length for the power-of-two grids the kernels are instantiated for, 0 otherwise
inline int static_len(int n)
{
	return (n == 64 || n == 128 || n == 256 || n == 512) ? n : 0;
}

// K2b in register form (mv_fft_y_reg): FP32 arithmetic, power-of-two gY up to 512 (E = 32 complex registers per
// component at 512, compiled for fewer resident blocks)
template <typename T> inline bool use_k2b_reg(int gY)
{
	return sizeof(T) == 4 && (gY == 64 || gY == 128 || gY == 256 || gY == 512);
}

// shared memory of a tile kernel for nl lines of length n: one tile in the column form (FP32, compile-time length),
// two for the Stockham passes
template <typename T> inline size_t tile_smem(int n, int nl)
{
	const bool one = sizeof(T) == 4 && static_len(n) != 0;
	// the column form's exchange buffer (lf_fft) needs E*(T*nl + pad) <= n*nl + 2n complex (pad < 16, E <= n/8)
	return one ? sizeof(typename CxT<T>::type) * (size_t)n * (tile_ls(nl) + 2)
		: 2 * sizeof(typename CxT<T>::type) * (size_t)n * tile_ls(nl);
}
// register K2b: NSLOT slots of BUF complex per lane group of T lanes
inline size_t k2b_reg_smem(int gY, int nt, bool surf)
{
	int lg = 0;
	while ((1 << lg) < gY) lg++;
	const int T = 1 << (lg / 2), E = gY / T;
	return (size_t)(nt / T) * (surf ? 4 : 3) * E * (T + 1) * sizeof(float2);
}
constexpr size_t SMEM_CAP = 216 * 1024; // dynamic shared memory of one block (the opt-in limit is 227 KB)

// Tile widths the build instantiates. The defaults (Tiles<T>) everywhere; for FP32 the tuner's alternatives (K1/K3 4
// y-lines; K2a/K2c 8 or 32; register K2b 64 or 256 threads; generic K2b 2 or 4 pairs) for every length; and, for the
// runtime-plan lengths
// (above 512 or not a power of two) the narrow tiles of long axes (1 y-line per K1/K3 block, 2 per K2a/K2c block,
// one (kz, RHS) pair per generic K2b block), whose shared memory fits axes up to 2048 (FP64) / 4096 (FP32).
template <typename T, int NS, int W> constexpr bool has_w1()
{
	return W == Tiles<T>::W1 || (sizeof(T) == 4 && W == 4) || (NS == 0 && W == 1);
}
template <typename T, int NS, int W> constexpr bool has_w2()
{
	return W == Tiles<T>::W2 || (sizeof(T) == 4 && (W == 8 || W == 32)) || (NS == 0 && W == 2);
}
template <typename T, int NS, int P> constexpr bool has_pairs()
{
	return P == Tiles<T>::PAIRS || (sizeof(T) == 4 && (P == 2 || P == 4)) || (NS == 0 && P == 1);
}
inline bool shape_instantiated(bool f32, int n1, int n2, int ny, const MvShape &s)
{
	const bool w1ok = s.w1 == (f32 ? 8 : 4) || (f32 && s.w1 == 4) || (static_len(n1) == 0 && s.w1 == 1);
	const bool w2ok = s.w2 == (f32 ? 16 : 8) || (f32 && (s.w2 == 8 || s.w2 == 32)) || (static_len(n2) == 0 && s.w2 == 2);
	const bool pok = s.pairs == (f32 ? 8 : 4) || (f32 && (s.pairs == 2 || s.pairs == 4)) ||
		(static_len(ny) == 0 && s.pairs == 1);
	const bool ntok = !f32 || s.nt == 64 || s.nt == 128 || s.nt == 256;
	return w1ok && w2ok && pok && ntok;
}
// the shared memory every kernel of the shape needs fits one block
template <typename T> inline bool shape_fits(const adda_gb300_ctx *c, const MvShape &s)
{
	if (tile_smem<T>(c->gX, 3 * s.w1) > SMEM_CAP || tile_smem<T>(c->gZ, s.w2) > SMEM_CAP) return false;
	if (use_k2b_reg<T>(c->gY)) return k2b_reg_smem(c->gY, s.nt, c->surface) <= SMEM_CAP;
	return 2 * sizeof(typename CxT<T>::type) * (size_t)c->gY * tile_ls(3 * s.pairs) <= SMEM_CAP && (!c->surface ||
		s.pairs >= 2);
}

#define ADDA_NS_SWITCH(n, CALL)                                                                                   \
	switch (static_len(n)) {                                                                                        \
		case 64: { constexpr int NS = 64; CALL; } break;                                                            \
		case 128: { constexpr int NS = 128; CALL; } break;                                                          \
		case 256: { constexpr int NS = 256; CALL; } break;                                                          \
		case 512: { constexpr int NS = 512; CALL; } break;                                                          \
		default: { constexpr int NS = 0; CALL; } break;                                                             \
	}
// one case per candidate width; CALL sees the width as the constant W (instantiated widths only)
#define ADDA_W_CASE(HAS, w, CALL)                                                                                   \
	case w: {                                                                                                       \
		if constexpr (HAS<T, NS, w>()) { constexpr int W = w; CALL; }                                               \
	} break;
#define ADDA_W_SWITCH(HAS, wv, CALL)                                                                                \
	switch (wv) {                                                                                                   \
		ADDA_W_CASE(HAS, 1, CALL) ADDA_W_CASE(HAS, 2, CALL) ADDA_W_CASE(HAS, 4, CALL) ADDA_W_CASE(HAS, 8, CALL)     \
		ADDA_W_CASE(HAS, 16, CALL) ADDA_W_CASE(HAS, 32, CALL)                                                       \
		default: break;                                                                                             \
	}

#define ADDA_SET(kern) ADDA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_CAP))
// shared-memory opt-in of the kernels that touch the dipole vectors (K1, K3)
template <typename T, typename V, int NS> int set_attrs_k13()
{
	for (int w : {1, 4, 8}) {
		ADDA_W_SWITCH(has_w1, w, ADDA_SET((mv_scatter_fftx<T, V, W, NS>)); ADDA_SET((mv_fftx_gather<T, V, W, NS>)))
	}
	return ADDA_GB300_OK;
}
// ... and of the y/z stage (K2a, K2b, K2c)
template <typename T, int NS> int set_attrs_yz()
{
	for (int w : {1, 2, 4, 8, 16, 32}) {
		ADDA_W_SWITCH(has_w2, w, ADDA_SET((mv_fftz<T, W, 0, NS>)); ADDA_SET((mv_fftz<T, W, 1, NS>));
			ADDA_SET((mv_fftz<T, W, 2, NS>)))
		ADDA_W_SWITCH(has_pairs, w, ADDA_SET((mv_fft_y_dmul<T, NS, W>)); ADDA_SET((mv_fft_y_surf<T, NS, W>)))
	}
	if constexpr (sizeof(T) == 4 && NS >= 64) {
		ADDA_SET((mv_fft_y_reg<NS, 64>));
		ADDA_SET((mv_fft_y_reg<NS, 128>));
		ADDA_SET((mv_fft_y_reg<NS, 256>));
		ADDA_SET((mv_fft_y_reg<NS, 64, true>));
		ADDA_SET((mv_fft_y_reg<NS, 128, true>));
		ADDA_SET((mv_fft_y_reg<NS, 256, true>));
	}
	return ADDA_GB300_OK;
}
#undef ADDA_SET

template <typename T, typename V> int set_attrs_tv()
{
	int rc;
	if ((rc = set_attrs_k13<T, V, 0>()) || (rc = set_attrs_k13<T, V, 64>()) || (rc = set_attrs_k13<T, V, 128>()) ||
		(rc = set_attrs_k13<T, V, 256>()) || (rc = set_attrs_k13<T, V, 512>()))
		return rc;
	return ADDA_GB300_OK;
}

template <typename T> int setup_yz()
{
	int rc;
	if ((rc = set_attrs_yz<T, 0>()) || (rc = set_attrs_yz<T, 64>()) || (rc = set_attrs_yz<T, 128>()) ||
		(rc = set_attrs_yz<T, 256>()) || (rc = set_attrs_yz<T, 512>()))
		return rc;
	return ADDA_GB300_OK;
}

// the y/z stage of one chunk of x-slabs (K2a, [K2a surface], K2b, K2c) with the context's tile shape, on stream st
template <typename T> int launch_yz(adda_gb300_ctx *c, MvGeom<T> p, int ck, const MvShape &sh, cudaStream_t st)
{
	const int R = p.R;
	const bool surf = c->surface;
	const dim3 g2((c->bY + sh.w2 - 1) / sh.w2, 3 * ck, R);
	ADDA_NS_SWITCH(c->gZ, ADDA_W_SWITCH(has_w2, sh.w2, (mv_fftz<T, W, 0, NS><<<g2, col_threads<T, NS, W>(),
		tile_smem<T>(c->gZ, W), st>>>(p))));
	ADDA_LAUNCHED();
	if (surf) {
		ADDA_NS_SWITCH(c->gZ, ADDA_W_SWITCH(has_w2, sh.w2, (mv_fftz<T, W, 2, NS><<<g2, col_threads<T, NS, W>(),
			tile_smem<T>(c->gZ, W), st>>>(p))));
		ADDA_LAUNCHED();
	}
	if (use_k2b_reg<T>(c->gY)) {
		if constexpr (sizeof(T) == 4) {
			const int nt = sh.nt;
			const int Tl = c->gY >= 256 ? 16 : 8; // lanes per line, RegShape<gY>::T
			const int G = nt / Tl;
			const dim3 g((c->gZ * R + G - 1) / G, ck);
			const size_t sm = k2b_reg_smem(c->gY, nt, surf);
#define ADDA_K2B_REG(NS_, NT_)                                                                                      \
	if (c->gY == NS_ && nt == NT_) {                                                                                \
		if (surf) mv_fft_y_reg<NS_, NT_, true><<<g, NT_, sm, st>>>(p);                                            \
		else mv_fft_y_reg<NS_, NT_><<<g, NT_, sm, st>>>(p);                                                       \
	}
			ADDA_K2B_REG(64, 64) ADDA_K2B_REG(64, 128) ADDA_K2B_REG(64, 256)
			ADDA_K2B_REG(128, 64) ADDA_K2B_REG(128, 128) ADDA_K2B_REG(128, 256)
			ADDA_K2B_REG(256, 64) ADDA_K2B_REG(256, 128) ADDA_K2B_REG(256, 256)
			ADDA_K2B_REG(512, 64) ADDA_K2B_REG(512, 128) ADDA_K2B_REG(512, 256)
#undef ADDA_K2B_REG
		}
	}
	else {
		// generic K2b: KB kz x RG RHS per block, KB*RG <= pairs (surface: pairs/2 six-line pairs)
		const int pairs = surf ? sh.pairs / 2 : sh.pairs;
		MvGeom<T> q = p;
		q.RG = std::min(R, pairs);
		q.KB = std::max(1, pairs / q.RG);
		const dim3 g2b((c->gZ + q.KB - 1) / q.KB, ck, (R + q.RG - 1) / q.RG);
		const size_t sm = 2 * sizeof(typename CxT<T>::type) * (size_t)c->gY * tile_ls(3 * sh.pairs);
		if (surf) {
			ADDA_NS_SWITCH(c->gY, ADDA_W_SWITCH(has_pairs, sh.pairs, (mv_fft_y_surf<T, NS, W><<<g2b, 256, sm, st>>>(q))));
		}
		else {
			ADDA_NS_SWITCH(c->gY, ADDA_W_SWITCH(has_pairs, sh.pairs, (mv_fft_y_dmul<T, NS, W><<<g2b, 256, sm, st>>>(q))));
		}
	}
	ADDA_LAUNCHED();
	ADDA_NS_SWITCH(c->gZ, ADDA_W_SWITCH(has_w2, sh.w2, (mv_fftz<T, W, 1, NS><<<g2, col_threads<T, NS, W>(),
		tile_smem<T>(c->gZ, W), st>>>(p))));
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

// the y/z stage and its set-up are compiled once per arithmetic, in matvec_yz.cu
#ifndef ADDA_MATVEC_YZ_TU
extern template int launch_yz<float>(adda_gb300_ctx *, MvGeom<float>, int, const MvShape &, cudaStream_t);
extern template int launch_yz<double>(adda_gb300_ctx *, MvGeom<double>, int, const MvShape &, cudaStream_t);
extern template int setup_yz<float>();
extern template int setup_yz<double>();
#endif

template <typename T, typename V>
int launch_matvec(adda_gb300_ctx *c, int R, const V *arg, V *res, int her, const MvEpi &epi, const int *done)
{
	typedef typename CxT<T>::type C;
	constexpr bool dbl = sizeof(T) == 8;
	const MvShape sh = c->shape[dbl ? 0 : 1];
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
	p.RG = p.KB = 1;
	p.TzR = (C *)c->TzR;
	p.Rm = dbl ? (const C *)c->R64 : (const C *)c->R32;
	p.RsY = c->gY / 2 + 1;
	p.rpp = c->rpp;
	p.lat_stride = c->lat_stride;
	cudaStream_t st = c->stream;
	const dim3 g1((c->bY + sh.w1 - 1) / sh.w1, c->bZ, R);
	ADDA_NS_SWITCH(c->gX, ADDA_W_SWITCH(has_w1, sh.w1, (mv_scatter_fftx<T, V, W, NS><<<g1, col_threads<T, NS, 3 * W>(),
		tile_smem<T>(c->gX, 3 * W), st>>>(p))));
	ADDA_LAUNCHED();
	// the y/z stage chunk by chunk, even chunks on the context stream with Tz, odd ones on the second stream with Tz2
	// (a chunk reuses its buffer only after the chunk two before it, on the same stream, has finished with it), so
	// that one chunk's kernels fill the other's tail; joined before K3
	int rc;
	const bool two = c->gX > p.CK;
	if (two) {
		ADDA_CUDA(cudaEventRecord(c->ev_fork, st));
		ADDA_CUDA(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
	}
	for (int kx0 = 0, i = 0; kx0 < c->gX; kx0 += p.CK, i++) {
		MvGeom<T> q = p;
		q.kx0 = kx0;
		if (i & 1) {
			q.Tz = (C *)c->Tz2;
			q.TzR = (C *)c->TzR2;
		}
		if ((rc = launch_yz<T>(c, q, std::min(p.CK, c->gX - kx0), sh, (i & 1) ? c->stream2 : st))) return rc;
	}
	if (two) {
		ADDA_CUDA(cudaEventRecord(c->ev_join, c->stream2));
		ADDA_CUDA(cudaStreamWaitEvent(st, c->ev_join, 0));
	}
	ADDA_NS_SWITCH(c->gX, ADDA_W_SWITCH(has_w1, sh.w1, (mv_fftx_gather<T, V, W, NS><<<g1, col_threads<T, NS, 3 * W>(),
		tile_smem<T>(c->gX, 3 * W), st>>>(p, epi))));
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

} // namespace mv
} // namespace adda
