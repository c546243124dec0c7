// dmatrix.cu - the interaction matrix D = -FFT(G)/Ngrid on the GPU in FP64 (InitDmatrix, src/fft.c:918-1416).
//
//   1. green_fill      : point-dipole Green's tensor (interaction.c:290-331) for every lattice offset
//                        (i in (-bX,bX), j in [0,bY), k in [0,bZ)), stored per component as [k][j][i mod gX]
//   2. fft_lines (x)   : forward FFT along x of every (component, k, j) line
//   3. per component   : slice_fill mirrors the (j,k) quarter into the full (y,z) plane of every kx with the
//                        parities of the tensor components (xy,yz odd in y; xz,yz odd in z; fft.c:1275-1290),
//                        fft_lines along z then y, and d_extract keeps y<=gY/2, z<=gZ/2 scaled by -1/Ngrid into the
//                        reduced layout [x][z][y][6] (fft.c:144-150, 1310-1314)
//   4. an FP32 copy for the single-precision matvec.
// This runs once per particle; it is written for clarity over speed (it costs a few FP64 3-D FFTs).
#include "ctx.cuh"

namespace adda {

namespace {

__global__ void green_fill(double2 *G, int bX, int bY, int bZ, int gX, double gridspace, double k)
{
	const size_t lines = (size_t)bZ * bY;
	const size_t total = lines * gX;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int xp = (int)(t % gX);
		const size_t jk = t / gX;
		const int j = (int)(jk % bY), kk = (int)(jk / bY);
		int i;
		bool valid = true;
		if (xp < bX) i = xp;
		else if (xp > gX - bX) i = xp - gX;
		else { i = 0; valid = false; }
		if (i == 0 && j == 0 && kk == 0) valid = false;
		double2 g[6];
		if (valid) {
			double q0 = i, q1 = j, q2 = kk;
			const double rn = sqrt(q0 * q0 + q1 * q1 + q2 * q2);
			const double invrn = 1.0 / rn;
			q0 *= invrn; q1 *= invrn; q2 *= invrn;
			const double rr = rn * gridspace;
			const double invr3 = 1 / (rr * rr * rr);
			const double kr = k * rr, kr2 = kr * kr;
			const double t1 = 3 - kr2, t2 = -3 * kr, t3 = kr2 - 1;
			double sn, cs;
			sincos(kr, &sn, &cs);
			const double evr = invr3 * cs, evi = invr3 * sn;
			const double qm[6] = {q0 * q0, q0 * q1, q0 * q2, q1 * q1, q1 * q2, q2 * q2};
#pragma unroll
			for (int a = 0; a < 6; a++) {
				double re, im;
				if (a == 0 || a == 3 || a == 5) {
					re = t1 * qm[a] + t3;
					im = kr + t2 * qm[a];
				}
				else {
					re = t1 * qm[a];
					im = t2 * qm[a];
				}
				g[a] = make_double2(re * evr - im * evi, re * evi + im * evr);
			}
		}
		else
			for (int a = 0; a < 6; a++) g[a] = make_double2(0, 0);
		for (int a = 0; a < 6; a++) G[(size_t)a * total + t] = g[a];
	}
}

// Generic batched FFT of lines: element e of line (o, l) at data[o*od + l*ls + e*es]. Blocks: x = tile of TL lines
// in l, y = o. Either es == 1 (contiguous lines) or ls == 1 (adjacent lines); tiles are loaded along that axis.
template <typename C>
__global__ void __launch_bounds__(256) fft_lines(C *data, FftPlan p, const C *__restrict__ tw, int inv, size_t es,
	size_t ls, int nl_inner, size_t od, int TL)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int LS = tile_ls(TL);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t)p.n * LS;
	const int n = p.n;
	const int l0 = blockIdx.x * TL;
	const int tl = min(TL, nl_inner - l0);
	C *base = data + blockIdx.y * od + (size_t)l0 * ls;
	const bool contig = (es == 1);
	for (int t = threadIdx.x; t < n * TL; t += blockDim.x) {
		int e, l;
		if (contig) { l = t / n; e = t % n; }
		else { e = t / TL; l = t % TL; }
		a[e * LS + l] = (l < tl) ? base[(size_t)l * ls + (size_t)e * es] : cx<C>(0, 0);
	}
	__syncthreads();
	C *o = fft_tile<C>(a, b, p, TL, LS, tw, inv != 0);
	for (int t = threadIdx.x; t < n * TL; t += blockDim.x) {
		int e, l;
		if (contig) { l = t / n; e = t % n; }
		else { e = t / TL; l = t % TL; }
		if (l < tl) base[(size_t)l * ls + (size_t)e * es] = o[e * LS + l];
	}
}

__global__ void slice_fill(double2 *S, const double2 *Ga, int bY, int bZ, int gX, int gY, int gZ, double sy,
	double sz)
{
	const size_t total = (size_t)gX * gY * gZ;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int z = (int)(t % gZ);
		const size_t xy = t / gZ;
		const int y = (int)(xy % gY), x = (int)(xy / gY);
		int j, kk;
		double s = 1;
		if (y < bY) j = y;
		else if (y > gY - bY) { j = gY - y; s *= sy; }
		else j = -1;
		if (z < bZ) kk = z;
		else if (z > gZ - bZ) { kk = gZ - z; s *= sz; }
		else kk = -1;
		double2 v = make_double2(0, 0);
		if (j >= 0 && kk >= 0) {
			const double2 g = Ga[((size_t)kk * bY + j) * gX + x];
			v = make_double2(s * g.x, s * g.y);
		}
		S[t] = v;
	}
}

__global__ void d_extract(double2 *D, const double2 *S, int a, int gX, int gY, int gZ, int DsY, int DsZ, double invN)
{
	const size_t total = (size_t)gX * DsZ * DsY;
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)(t % DsY);
		const size_t xz = t / DsY;
		const int z = (int)(xz % DsZ), x = (int)(xz / DsZ);
		const double2 v = S[((size_t)x * gY + y) * gZ + z];
		D[t * 6 + a] = make_double2(-invN * v.x, -invN * v.y);
	}
}

__global__ void to_f32(float2 *dst, const double2 *src, size_t n)
{
	for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
		dst[t] = make_float2((float)src[t].x, (float)src[t].y);
}

int grid_for(size_t n)
{
	size_t g = (n + 255) / 256;
	if (g > 152 * 64) g = 152 * 64;
	if (g < 1) g = 1;
	return (int)g;
}

// FFT of all lines described by (es, ls, nl_inner, od, nouter) with the FP64 plan p
int fft_lines_run(adda_gb300_ctx *c, double2 *data, const FftPlan &p, const double2 *tw, bool inv, size_t es,
	size_t ls, int nl_inner, size_t od, int nouter)
{
	int TL = 16;
	while (TL > 1 && 2 * sizeof(double2) * (size_t)p.n * tile_ls(TL) > 200 * 1024) TL /= 2;
	const size_t smem = 2 * sizeof(double2) * (size_t)p.n * tile_ls(TL);
	ADDA_CUDA(cudaFuncSetAttribute(fft_lines<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	dim3 g((nl_inner + TL - 1) / TL, nouter);
	fft_lines<double2><<<g, 256, smem, c->stream>>>(data, p, tw, inv ? 1 : 0, es, ls, nl_inner, od, TL);
	ADDA_LAUNCHED();
	return ADDA_GB300_OK;
}

} // namespace

int dmatrix_build(adda_gb300_ctx *c)
{
	const int bX = c->bX, bY = c->bY, bZ = c->bZ, gX = c->gX, gY = c->gY, gZ = c->gZ;
	const size_t lines = (size_t)bZ * bY;
	const size_t gsz = lines * gX;
	const size_t ssz = (size_t)gX * gY * gZ;
	const size_t dlen = (size_t)gX * c->DsZ * c->DsY * 6;
	double2 *G = nullptr, *S = nullptr;
	int rc = ADDA_GB300_OK;
	if (cudaMalloc(&G, sizeof(double2) * 6 * gsz) != cudaSuccess ||
		cudaMalloc(&S, sizeof(double2) * ssz) != cudaSuccess) {
		cudaFree(G);
		set_error("cannot allocate the D-matrix build buffers");
		return ADDA_GB300_ENOMEM;
	}
	const double invN = 1.0 / (gX * ((double)gY * gZ));
	do {
		green_fill<<<grid_for(gsz), 256, 0, c->stream>>>(G, bX, bY, bZ, gX, c->gridspace, c->k);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		// x transform of all 6*bZ*bY lines (contiguous, length gX)
		if ((rc = fft_lines_run(c, G, c->px[0], c->tw64[0], false, 1, gX, (int)(6 * lines), 0, 1))) break;
		for (int a = 0; a < 6 && !rc; a++) {
			const double sy = (a == 1 || a == 4) ? -1 : 1, sz = (a == 2 || a == 4) ? -1 : 1;
			slice_fill<<<grid_for(ssz), 256, 0, c->stream>>>(S, G + (size_t)a * gsz, bY, bZ, gX, gY, gZ, sy, sz);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
			// z transform: lines (x,y) contiguous of length gZ
			if ((rc = fft_lines_run(c, S, c->pz[0], c->tw64[2], false, 1, gZ, gX * gY, 0, 1))) break;
			// y transform: element stride gZ, lines z adjacent, outer x
			if ((rc = fft_lines_run(c, S, c->py[0], c->tw64[1], false, gZ, 1, gZ, (size_t)gY * gZ, gX))) break;
			d_extract<<<grid_for((size_t)gX * c->DsZ * c->DsY), 256, 0, c->stream>>>(c->D64, S, a, gX, gY, gZ,
				c->DsY, c->DsZ, invN);
			count_launch();
			if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		}
		if (rc) break;
		to_f32<<<grid_for(dlen), 256, 0, c->stream>>>(c->D32, c->D64, dlen);
		count_launch();
		if (cudaGetLastError() != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
		if (cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = ADDA_GB300_ECUDA; break; }
	} while (0);
	if (rc == ADDA_GB300_ECUDA) set_error(std::string("D-matrix build: ") + cudaGetErrorString(cudaGetLastError()));
	cudaFree(G);
	cudaFree(S);
	if (!rc) c->dready = true;
	return rc;
}

} // namespace adda
