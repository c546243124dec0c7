// common.cuh - complex arithmetic, FFT plans and the shared-memory tile FFT used by every kernel of the library.
//
// The tile FFT transforms nl lines of length n held in shared memory in ELEMENT-MAJOR order (element e of line l at
// a[e*ls + l], ls = odd stride >= nl): consecutive threads work on consecutive lines, so every pass is conflict-free,
// and the odd stride also keeps the element-strided accesses of the load/store phases conflict-free (an 8-byte
// element at an odd stride visits every bank pair once per 16 threads). Tiles gathered from HBM along the contiguous
// axis of the data need no transpose. Each pass is a
// self-sorting Stockham radix-R step (ping-pong between two tiles); radices 2,3,4,8,16 are hand-written register
// butterflies, 5/7/11/13 a symmetric-pair register butterfly (dft_odd). Twiddles come from one table of n-th roots of unity per length, computed on the
// host in double precision. Sign convention: forward = exp(-2*pi*i*jk/n), unnormalised, like FFTW's FFTW_FORWARD
// which the reference uses (fft.h FFT_FORWARD -1).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace adda {

template <typename T> struct CxT;
template <> struct CxT<float> { typedef float2 type; };
template <> struct CxT<double> { typedef double2 type; };

template <typename C> __host__ __device__ __forceinline__ C cx(decltype(C::x) a, decltype(C::x) b)
{
	C r;
	r.x = a;
	r.y = b;
	return r;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return cx<C>(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return cx<C>(a.x - b.x, a.y - b.y); }
// Pairs of floats. Sums run on Blackwell's packed FP32 pipe: add/sub.rn.f32x2 process both halves in one issue slot,
// each half rounded to nearest like the scalar instruction (never contracted: the error-free transformations of the
// double-float code below rely on it). A complex float2 sum is one instruction, which halves the issue slots of the
// FFT butterflies (mostly such sums) and of the double-float complex arithmetic. Built with -DADDA_NO_F32X2 the sums
// are scalar __fadd_rn/__fsub_rn, which must give the same bits (the tests compare the two builds). Scalar on the
// host.
#if defined(__CUDA_ARCH__) && !defined(ADDA_NO_F32X2)
#define ADDA_F32X2 1
__device__ __forceinline__ unsigned long long f2_bits(float2 a)
{
	unsigned long long r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
	return r;
}
__device__ __forceinline__ float2 f2_of(unsigned long long r)
{
	float2 a;
	asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
	return a;
}
#endif
__host__ __device__ __forceinline__ float2 p_add(float2 a, float2 b)
{
#ifdef ADDA_F32X2
	unsigned long long r;
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
	return f2_of(r);
#elif defined(__CUDA_ARCH__)
	return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
#else
	return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 p_sub(float2 a, float2 b)
{
#ifdef ADDA_F32X2
	unsigned long long r;
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
	return f2_of(r);
#elif defined(__CUDA_ARCH__)
	return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
#else
	return make_float2(a.x - b.x, a.y - b.y);
#endif
}
// products stay scalar round-to-nearest operations: a packed mul.f32x2 did not give the scalar instruction's bits in
// every compiled context (a bit-for-bit check against __fmul_rn found differences inside larger kernels), so only the
// sums, which do, use the packed pipe
__host__ __device__ __forceinline__ float2 p_mul(float2 a, float2 b)
{
#ifdef __CUDA_ARCH__
	return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
#else
	return make_float2(a.x * b.x, a.y * b.y);
#endif
}
// a*b + c per half, one rounding
__host__ __device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c)
{
#ifdef __CUDA_ARCH__
	return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
#else
	return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return p_add(a, b); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return p_sub(a, b); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b)
{
	return cx<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { return cx<C>(a.x, -a.y); }
template <typename C> __host__ __device__ __forceinline__ C cneg(C a) { return cx<C>(-a.x, -a.y); }
template <typename C, typename S> __host__ __device__ __forceinline__ C cscale(C a, S s)
{
	return cx<C>(a.x * s, a.y * s);
}
// a*b + c
template <typename C> __host__ __device__ __forceinline__ C cfma(C a, C b, C c)
{
	return cx<C>(a.x * b.x - a.y * b.y + c.x, a.x * b.y + a.y * b.x + c.y);
}
__host__ __device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(a.x, a.y); }
__host__ __device__ __forceinline__ double2 to_d2(double2 a) { return a; }
template <typename C> __host__ __device__ __forceinline__ C from_d2(double2 a);
template <> __host__ __device__ __forceinline__ float2 from_d2<float2>(double2 a)
{
	return make_float2((float)a.x, (float)a.y);
}
template <> __host__ __device__ __forceinline__ double2 from_d2<double2>(double2 a) { return a; }

// ---------------------------------------------------------------------------------------------------------------
// Double-float numbers: the unevaluated sum h + l of two floats with |l| <= ulp(h)/2 (about 48 significant bits),
// computed on the FP32 pipes with error-free transformations: TwoSum (Knuth), FastTwoSum (Dekker) and the exact
// product error through FMA; addition and multiplication follow the double-double algorithms of Dekker (1971) as
// used in Bailey's QD library, with floats in place of doubles (addition in its "sloppy" form: error bounded by a
// few 2^-48 of the operands). GB300 executes FP64 at about 1/64 of its FP32 rate, so Krylov vectors held in this
// form update at memory speed. The __f*_rn intrinsics are never contracted into FMAs, which the transformations
// rely on.
struct DF {
	float h, l;
};

__host__ __device__ __forceinline__ DF df_two_sum(float a, float b)
{
#ifdef __CUDA_ARCH__
	const float s = __fadd_rn(a, b), v = __fsub_rn(s, a);
	return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
#else
	const float s = a + b, v = s - a;
	return DF{s, (a - (s - v)) + (b - v)};
#endif
}
__host__ __device__ __forceinline__ DF df_fast_two_sum(float a, float b) // |a| >= |b|
{
#ifdef __CUDA_ARCH__
	const float s = __fadd_rn(a, b);
	return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
#else
	const float s = a + b;
	return DF{s, b - (s - a)};
#endif
}
__host__ __device__ __forceinline__ DF operator+(DF a, DF b)
{
	const DF s = df_two_sum(a.h, b.h);
#ifdef __CUDA_ARCH__
	return df_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
#else
	return df_fast_two_sum(s.h, s.l + (a.l + b.l));
#endif
}
__host__ __device__ __forceinline__ DF operator-(DF a) { return DF{-a.h, -a.l}; }
__host__ __device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__host__ __device__ __forceinline__ DF operator*(DF a, DF b)
{
#ifdef __CUDA_ARCH__
	const float p = __fmul_rn(a.h, b.h);
	float e = __fmaf_rn(a.h, b.h, -p);
	e = __fmaf_rn(a.h, b.l, e);
	e = __fmaf_rn(a.l, b.h, e);
	return df_fast_two_sum(p, e);
#else
	const double p = (double)a.h * b.h + (double)a.h * b.l + (double)a.l * b.h;
	const float h = (float)p;
	return DF{h, (float)(p - h)};
#endif
}
__host__ __device__ __forceinline__ DF df_of(double v)
{
	const float h = (float)v;
	return DF{h, (float)(v - (double)h)};
}
__host__ __device__ __forceinline__ double df_val(DF a) { return (double)a.h + (double)a.l; }

// complex double-float: the Krylov vector element of the MIXED solver (16 bytes, like double2). The high parts of
// the real and imaginary part share one float2, the low parts the other, so that the double-float arithmetic of a
// complex value runs on packed FP32 pairs (both parts in one instruction).
struct __align__(16) dd2 {
	float2 h, l; // re = h.x + l.x, im = h.y + l.y
};
__host__ __device__ __forceinline__ DF dd2_re(dd2 a) { return DF{a.h.x, a.l.x}; }
__host__ __device__ __forceinline__ DF dd2_im(dd2 a) { return DF{a.h.y, a.l.y}; }
__host__ __device__ __forceinline__ dd2 make_dd2(DF re, DF im)
{
	return dd2{make_float2(re.h, im.h), make_float2(re.l, im.l)};
}
__host__ __device__ __forceinline__ double2 to_d2(dd2 a) { return make_double2(df_val(dd2_re(a)), df_val(dd2_im(a))); }
template <> __host__ __device__ __forceinline__ dd2 from_d2<dd2>(double2 a) { return make_dd2(df_of(a.x), df_of(a.y)); }

// Packed double-float arithmetic: the scalar algorithms above applied to the two halves at once.
// TwoSum of each half: s + e = a + b exactly
__host__ __device__ __forceinline__ void p_two_sum(float2 a, float2 b, float2 &s, float2 &e)
{
	s = p_add(a, b);
	const float2 v = p_sub(s, a);
	e = p_add(p_sub(a, p_sub(s, v)), p_sub(b, v));
}
// s + e = a - b exactly
__host__ __device__ __forceinline__ void p_two_diff(float2 a, float2 b, float2 &s, float2 &e)
{
	s = p_sub(a, b);
	const float2 v = p_sub(s, a);
	e = p_sub(p_sub(a, p_sub(s, v)), p_add(b, v));
}
// renormalisation (FastTwoSum, |a| >= |b| per half)
__host__ __device__ __forceinline__ dd2 p_renorm(float2 a, float2 b)
{
	const float2 s = p_add(a, b);
	return dd2{s, p_sub(b, p_sub(s, a))};
}
__host__ __device__ __forceinline__ dd2 cadd(dd2 a, dd2 b)
{
	float2 s, e;
	p_two_sum(a.h, b.h, s, e);
	return p_renorm(s, p_add(e, p_add(a.l, b.l)));
}
__host__ __device__ __forceinline__ dd2 csub(dd2 a, dd2 b)
{
	float2 s, e;
	p_two_diff(a.h, b.h, s, e);
	return p_renorm(s, p_add(e, p_sub(a.l, b.l)));
}
// elementwise product of the halves: (a.re*b.re, a.im*b.im) as double-floats; exact product error through FMA
__host__ __device__ __forceinline__ dd2 p_hmul(dd2 a, dd2 b)
{
	const float2 p = p_mul(a.h, b.h);
	float2 e = p_fma(a.h, b.h, p_sub(make_float2(0.f, 0.f), p));
	e = p_fma(a.h, b.l, e);
	e = p_fma(a.l, b.h, e);
	return p_renorm(p, e);
}
__host__ __device__ __forceinline__ dd2 dd2_swap(dd2 a)
{
	return dd2{make_float2(a.h.y, a.h.x), make_float2(a.l.y, a.l.x)};
}
__host__ __device__ __forceinline__ dd2 cconj(dd2 a)
{
	return dd2{make_float2(a.h.x, -a.h.y), make_float2(a.l.x, -a.l.y)};
}
__host__ __device__ __forceinline__ dd2 cneg(dd2 a) { return dd2{make_float2(-a.h.x, -a.h.y), make_float2(-a.l.x, -a.l.y)}; }
// real double-float factor
__host__ __device__ __forceinline__ dd2 cscale(dd2 a, DF s)
{
	return p_hmul(a, dd2{make_float2(s.h, s.h), make_float2(s.l, s.l)});
}
// a*b = (a.re b.re - a.im b.im, a.re b.im + a.im b.re) = a.re*(b.re, b.im) + a.im*(-b.im, b.re)
__host__ __device__ __forceinline__ dd2 cmul(dd2 a, dd2 b)
{
	const dd2 ar{make_float2(a.h.x, a.h.x), make_float2(a.l.x, a.l.x)};
	const dd2 ai{make_float2(-a.h.y, a.h.y), make_float2(-a.l.y, a.l.y)};
	return cadd(p_hmul(ar, b), p_hmul(ai, dd2_swap(b)));
}
// a loop-invariant complex factor k prepared once: k*v = (k.re, k.re)*(v.re, v.im) + (-k.im, k.im)*(v.im, v.re)
struct dd2k {
	dd2 re, im;
};
__host__ __device__ __forceinline__ dd2k make_dd2k(dd2 k)
{
	return dd2k{dd2{make_float2(k.h.x, k.h.x), make_float2(k.l.x, k.l.x)},
		dd2{make_float2(-k.h.y, k.h.y), make_float2(-k.l.y, k.l.y)}};
}
__host__ __device__ __forceinline__ dd2 cmul(dd2k k, dd2 v) { return cadd(p_hmul(k.re, v), p_hmul(k.im, dd2_swap(v))); }
__host__ __device__ __forceinline__ dd2 cmul(dd2 v, dd2k k) { return cmul(k, v); }

// real coefficient in the arithmetic of the vector type C
template <typename C> struct RealOf {
	typedef decltype(C::x) T;
	static __host__ __device__ __forceinline__ T make(double v) { return (T)v; }
};
template <> struct RealOf<dd2> {
	typedef DF T;
	static __host__ __device__ __forceinline__ DF make(double v) { return df_of(v); }
};
template <typename C> __host__ __device__ __forceinline__ typename RealOf<C>::T rof(double v) { return RealOf<C>::make(v); }

// Per-thread accumulators of the fused reductions: double for float2/double2 vectors (exact products of floats,
// FP64 sums), double-float for dd2 vectors (no FP64 instruction per element). acc_val gives the double the block
// reductions continue with.
template <typename C> struct AccOf {
	typedef double T;
};
template <> struct AccOf<dd2> {
	typedef DF T;
};
__host__ __device__ __forceinline__ double acc_val(double a) { return a; }
__host__ __device__ __forceinline__ double acc_val(DF a) { return df_val(a); }
// s += |y|^2
template <typename C> __device__ __forceinline__ void acc_abs2(double &s, C y)
{
	const double2 d = to_d2(y);
	s += d.x * d.x + d.y * d.y;
}
__device__ __forceinline__ void acc_abs2(DF &s, dd2 y)
{
	const dd2 q = p_hmul(y, y); // (re^2, im^2)
	s = s + (dd2_re(q) + dd2_im(q));
}
// (sr, si) += a*b
template <typename C> __device__ __forceinline__ void acc_cmul(double &sr, double &si, C a, C b)
{
	const double2 x = to_d2(a), y = to_d2(b);
	sr += x.x * y.x - x.y * y.y;
	si += x.x * y.y + x.y * y.x;
}
__device__ __forceinline__ void acc_cmul(DF &sr, DF &si, dd2 a, dd2 b)
{
	const dd2 p = p_hmul(a, b), q = p_hmul(a, dd2_swap(b)); // (re*re, im*im), (re*im, im*re)
	sr = sr + (dd2_re(p) - dd2_im(p));
	si = si + (dd2_re(q) + dd2_im(q));
}
// (sr, si) += a*conj(b)
template <typename C> __device__ __forceinline__ void acc_cmulc(double &sr, double &si, C a, C b)
{
	const double2 x = to_d2(a), y = to_d2(b);
	sr += x.x * y.x + x.y * y.y;
	si += x.y * y.x - x.x * y.y;
}
__device__ __forceinline__ void acc_cmulc(DF &sr, DF &si, dd2 a, dd2 b)
{
	const dd2 p = p_hmul(a, b), q = p_hmul(a, dd2_swap(b)); // (re*re, im*im), (re*im, im*re)
	sr = sr + (dd2_re(p) + dd2_im(p));
	si = si + (dd2_im(q) - dd2_re(q));
}
// s[0] += Re(y)^2, s[1] += Im(y)^2, s[2] += Re(y)*Im(y)
template <typename C> __device__ __forceinline__ void acc_sq3(double *s, C y)
{
	const double2 d = to_d2(y);
	s[0] += d.x * d.x;
	s[1] += d.y * d.y;
	s[2] += d.x * d.y;
}
__device__ __forceinline__ void acc_sq3(DF *s, dd2 y)
{
	const dd2 q = p_hmul(y, y), r = p_hmul(y, dd2_swap(y)); // (re^2, im^2), (re*im, im*re)
	s[0] = s[0] + dd2_re(q);
	s[1] = s[1] + dd2_im(q);
	s[2] = s[2] + dd2_re(r);
}

// ---------------------------------------------------------------------------------------------------------------
// FFT plan: the radix of each Stockham pass. Filled on the host (make_plan in api.cu), passed to kernels by value.
#define ADDA_FFT_MAXPASS 12
struct FftPlan {
	int n;
	int np;
	int r[ADDA_FFT_MAXPASS];
};

// multiply by exp(s*i*theta) given c=cos(theta), s_=s*sin(theta)
template <typename C> __device__ __forceinline__ C crot(C v, double c, double s_)
{
	typedef decltype(C::x) T;
	return cx<C>(v.x * (T)c - v.y * (T)s_, v.x * (T)s_ + v.y * (T)c);
}
// multiply by -i (forward) or +i (inverse)
template <typename C> __device__ __forceinline__ C cmi(C v, bool inv) { return inv ? cx<C>(-v.y, v.x) : cx<C>(v.y, -v.x); }

template <typename C> __device__ __forceinline__ void dft2(C &a, C &b)
{
	C t = a;
	a = cadd(t, b);
	b = csub(t, b);
}

template <typename C> __device__ __forceinline__ void dft4(C *v, bool inv)
{
	C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
	C t2 = cadd(v[1], v[3]), t3 = cmi(csub(v[1], v[3]), inv);
	v[0] = cadd(t0, t2);
	v[2] = csub(t0, t2);
	v[1] = cadd(t1, t3);
	v[3] = csub(t1, t3);
}

// radix-8 as two radix-4 halves (even/odd inputs) joined by W8^k
template <typename C> __device__ __forceinline__ void dft8(C *v, bool inv)
{
	const double h = 0.70710678118654752440; // sqrt(2)/2
	const double sg = inv ? 1.0 : -1.0;
	C e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
	dft4(e, inv);
	dft4(o, inv);
	o[1] = crot(o[1], h, sg * h);
	o[2] = cmi(o[2], inv);
	o[3] = crot(o[3], -h, sg * h);
#pragma unroll
	for (int k = 0; k < 4; k++) {
		v[k] = cadd(e[k], o[k]);
		v[k + 4] = csub(e[k], o[k]);
	}
}

// radix-16 as two radix-8 halves joined by W16^k
template <typename C> __device__ __forceinline__ void dft16(C *v, bool inv)
{
	const double c1 = 0.92387953251128675613, s1 = 0.38268343236508977173, h = 0.70710678118654752440;
	const double sg = inv ? 1.0 : -1.0;
	C e[8], o[8];
#pragma unroll
	for (int q = 0; q < 8; q++) {
		e[q] = v[2 * q];
		o[q] = v[2 * q + 1];
	}
	dft8(e, inv);
	dft8(o, inv);
	o[1] = crot(o[1], c1, sg * s1);
	o[2] = crot(o[2], h, sg * h);
	o[3] = crot(o[3], s1, sg * c1);
	o[4] = cmi(o[4], inv);
	o[5] = crot(o[5], -s1, sg * c1);
	o[6] = crot(o[6], -h, sg * h);
	o[7] = crot(o[7], -c1, sg * s1);
#pragma unroll
	for (int k = 0; k < 8; k++) {
		v[k] = cadd(e[k], o[k]);
		v[k + 8] = csub(e[k], o[k]);
	}
}

// radix-32 as two radix-16 halves joined by W32^k (k = 0..15)
template <typename C> __device__ __forceinline__ void dft32(C *v, bool inv)
{
	const double sg = inv ? 1.0 : -1.0;
	C e[16], o[16];
#pragma unroll
	for (int q = 0; q < 16; q++) {
		e[q] = v[2 * q];
		o[q] = v[2 * q + 1];
	}
	dft16(e, inv);
	dft16(o, inv);
	// cos/sin(k*pi/16), k = 1..7
	const double c[8] = {1.0, 0.98078528040323044913, 0.92387953251128675613, 0.83146961230254523708,
		0.70710678118654752440, 0.55557023301960222474, 0.38268343236508977173, 0.19509032201612826785};
#pragma unroll
	for (int k = 1; k < 16; k++) {
		// angle k*pi/16: cos = c[k] for k<8, -c[16-k] for k>8; sin = c[8-k] for k<=8, c[k-8] for k>8
		const double cs = (k < 8) ? c[k] : (k == 8 ? 0.0 : -c[16 - k]);
		const double sn = (k <= 8) ? (k == 8 ? 1.0 : c[8 - k]) : c[k - 8];
		o[k] = crot(o[k], cs, sg * sn);
	}
#pragma unroll
	for (int k = 0; k < 16; k++) {
		v[k] = cadd(e[k], o[k]);
		v[k + 16] = csub(e[k], o[k]);
	}
}

template <typename C> __device__ __forceinline__ void dft3(C *v, bool inv)
{
	typedef decltype(C::x) T;
	const T s = (T)(inv ? 0.86602540378443864676 : -0.86602540378443864676);
	C t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
	C m1 = cx<C>(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
	C m2 = cx<C>(-s * t2.y, s * t2.x); // i*s*t2
	v[0] = cadd(v[0], t1);
	v[1] = cadd(m1, m2);
	v[2] = csub(m1, m2);
}

// cos/sin(2*pi*k/R), k = 0..(R-1)/2, for the odd prime radices of fftFit's sizes (local constant tables: with the
// index known after unrolling they fold into immediates)
template <int R> __device__ __forceinline__ double odd_cos(int k)
{
	if constexpr (R == 5) {
		const double t[3] = {1.0, 0.30901699437494745126, -0.80901699437494734024};
		return t[k];
	}
	else if constexpr (R == 7) {
		const double t[4] = {1.0, 0.62348980185873359439, -0.22252093395631433737, -0.90096886790241903498};
		return t[k];
	}
	else if constexpr (R == 11) {
		const double t[6] = {1.0, 0.84125353283118120551, 0.41541501300188643508, -0.14231483827328500480,
			-0.65486073394528498959, -0.95949297361449736865};
		return t[k];
	}
	else {
		const double t[7] = {1.0, 0.88545602565320991051, 0.56806474673115592289, 0.12053668025532300601,
			-0.35460488704253545489, -0.74851074817110119231, -0.97094181742605201180};
		return t[k];
	}
}
template <int R> __device__ __forceinline__ double odd_sin(int k)
{
	if constexpr (R == 5) {
		const double t[3] = {0.0, 0.95105651629515353118, 0.58778525229247324813};
		return t[k];
	}
	else if constexpr (R == 7) {
		const double t[4] = {0.0, 0.78183148246802980363, 0.97492791218182361934, 0.43388373911755823142};
		return t[k];
	}
	else if constexpr (R == 11) {
		const double t[6] = {0.0, 0.54064081745559755543, 0.90963199535451833011, 0.98982144188093279524,
			0.75574957435425826890, 0.28173255684142967104};
		return t[k];
	}
	else {
		const double t[7] = {0.0, 0.46472317204376850652, 0.82298386589365635224, 0.99270887409805397272,
			0.93501624268541483342, 0.66312265824079519305, 0.23931566428755768339};
		return t[k];
	}
}

// DFT of odd prime length R in registers, symmetric-pair form: with a_p = x_p + x_(R-p), b_p = x_p - x_(R-p),
// X_k = x_0 + sum_p a_p cos(2 pi p k / R) -/+ i sum_p b_p sin(2 pi p k / R) and X_(R-k) with the other sign
// ((R-1)^2 real multiply-adds instead of the R^2 complex ones of the direct sum).
template <typename C, int R> __device__ __forceinline__ void dft_odd(C *v, bool inv)
{
	typedef decltype(C::x) T;
	constexpr int H = (R - 1) / 2;
	C a[H], b[H];
#pragma unroll
	for (int p = 1; p <= H; p++) {
		a[p - 1] = cadd(v[p], v[R - p]);
		b[p - 1] = csub(v[p], v[R - p]);
	}
	const C x0 = v[0];
	C sum = x0;
#pragma unroll
	for (int p = 0; p < H; p++) sum = cadd(sum, a[p]);
	v[0] = sum;
#pragma unroll
	for (int k = 1; k <= H; k++) {
		C t = x0, u = cx<C>(0, 0);
#pragma unroll
		for (int p = 1; p <= H; p++) {
			const int i = (p * k) % R;
			const T cs = (T)(i <= H ? odd_cos<R>(i) : odd_cos<R>(R - i));
			const T sn = (T)(i <= H ? odd_sin<R>(i) : -odd_sin<R>(R - i));
			t.x += cs * a[p - 1].x;
			t.y += cs * a[p - 1].y;
			u.x += sn * b[p - 1].x;
			u.y += sn * b[p - 1].y;
		}
		// forward: X_k = t - i u, X_(R-k) = t + i u; inverse the other way round
		const C m = cx<C>(t.x + u.y, t.y - u.x), q = cx<C>(t.x - u.y, t.y + u.x);
		v[k] = inv ? q : m;
		v[R - k] = inv ? m : q;
	}
}

template <typename C, int R> __device__ __forceinline__ void dft(C *v, bool inv, const C *__restrict__ tw, int n)
{
	if constexpr (R == 2) dft2(v[0], v[1]);
	else if constexpr (R == 3) dft3(v, inv);
	else if constexpr (R == 4) dft4(v, inv);
	else if constexpr (R == 8) dft8(v, inv);
	else if constexpr (R == 16) dft16(v, inv);
	else if constexpr (R == 32) dft32(v, inv);
	else if constexpr (R == 5 || R == 7 || R == 11 || R == 13) dft_odd<C, R>(v, inv);
}

// v * exp(-/+ i k pi/16) (forward / inverse), k in [0, 16): k is a constant after unrolling, so every branch folds
template <typename C> __device__ __forceinline__ C rot_pi16(C v, int k, bool inv)
{
	// cos(k pi/16), k = 0..8
	const double c[9] = {1.0, 0.98078528040323044913, 0.92387953251128675613, 0.83146961230254523708,
		0.70710678118654752440, 0.55557023301960222474, 0.38268343236508977173, 0.19509032201612826785, 0.0};
	const double sg = inv ? 1.0 : -1.0;
	if (k == 0) return v;
	if (k == 8) return cmi(v, inv);
	const double cs = k < 8 ? c[k] : -c[16 - k];
	const double sn = k < 8 ? c[8 - k] : c[k - 8];
	return crot(v, cs, sg * sn);
}

// DFT of length R (8, 16 or 32) of a line whose upper half is zero (v[j] = 0 for j >= R/2; those registers are not
// read): X[2m] = DFT_(R/2)(x)[m] and X[2m+1] = DFT_(R/2)(x_j W_R^j)[m]. Every zero-padded transform of the matvec
// starts like this (an axis of the FFT grid is at least twice the particle's), and it saves the R complex sums of
// the full transform's last stage.
template <typename C, int R> __device__ __forceinline__ void dft_half_in(C *v, bool inv)
{
	constexpr int H = R / 2;
	C e[H], o[H];
#pragma unroll
	for (int j = 0; j < H; j++) {
		e[j] = v[j];
		o[j] = rot_pi16(v[j], j * (32 / R), inv);
	}
	dft<C, H>(e, inv, nullptr, R);
	dft<C, H>(o, inv, nullptr, R);
#pragma unroll
	for (int m = 0; m < H; m++) {
		v[2 * m] = e[m];
		v[2 * m + 1] = o[m];
	}
}

// One Stockham pass over all lines of an element-major tile: x -> y.
template <typename C, int R>
__device__ __forceinline__ void fft_pass(const C *__restrict__ x, C *__restrict__ y, int n, int nl, int ls, int m,
	const C *__restrict__ tw, bool inv)
{
	const int nr = n / R;
	const int total = nr * nl;
	const int tstep = n / (m * R);
	for (int w = threadIdx.x; w < total; w += blockDim.x) {
		const int j = w / nl;
		const int l = w - j * nl;
		const int k = j % m;
		C v[R];
#pragma unroll
		for (int q = 0; q < R; q++) v[q] = x[(j + q * nr) * ls + l];
		if (k) {
#pragma unroll
			for (int q = 1; q < R; q++) {
				C t = __ldg(tw + q * k * tstep);
				if (inv) t.y = -t.y;
				v[q] = cmul(v[q], t);
			}
		}
		dft<C, R>(v, inv, tw, n);
		const int base = (j / m) * m * R + k;
#pragma unroll
		for (int q = 0; q < R; q++) y[(base + q * m) * ls + l] = v[q];
	}
}

// Stockham pass for the rarer odd radices 5,7,11,13 (fftFit sizes): O(R^2) with both twiddle factors folded into
// one table lookup, tw[(p*k*(n/(m*R)) + (q*p mod R)*(n/R)) mod n]; loops instead of register arrays keep the register
// footprint of the hot radix-2^k kernels low.
template <typename C>
__device__ __noinline__ void fft_pass_gen(const C *__restrict__ x, C *__restrict__ y, int R, int n, int nl, int ls,
	int m, const C *__restrict__ tw, bool inv)
{
	const int nr = n / R;
	const int total = nr * nl;
	const int tstep = n / (m * R);
	const int st = n / R;
	for (int w = threadIdx.x; w < total; w += blockDim.x) {
		const int j = w / nl;
		const int l = w - j * nl;
		const int k = j % m;
		const int base = (j / m) * m * R + k;
		for (int q = 0; q < R; q++) {
			C acc = cx<C>(0, 0);
			for (int p = 0; p < R; p++) {
				const int e = (p * k * tstep + ((q * p) % R) * st) % n;
				C t = __ldg(tw + e);
				if (inv) t.y = -t.y;
				acc = cfma(x[(j + p * nr) * ls + l], t, acc);
			}
			y[(base + q * m) * ls + l] = acc;
		}
	}
}

// odd line stride for an element-major tile of nl lines
__host__ __device__ constexpr int tile_ls(int nl) { return nl | 1; }

// Full FFT of an element-major tile (n elements x nl lines, stride ls) in a, using b as scratch. Returns the buffer
// holding the result (a or b). All threads of the block must call it; it synchronises between passes and at the end.
template <typename C>
__device__ C *fft_tile(C *a, C *b, const FftPlan &p, int nl, int ls, const C *__restrict__ tw, bool inv)
{
	const int n = p.n;
	int m = 1;
	for (int f = 0; f < p.np; f++) {
		const int R = p.r[f];
		switch (R) {
			case 2: fft_pass<C, 2>(a, b, n, nl, ls, m, tw, inv); break;
			case 3: fft_pass<C, 3>(a, b, n, nl, ls, m, tw, inv); break;
			case 4: fft_pass<C, 4>(a, b, n, nl, ls, m, tw, inv); break;
			case 8: fft_pass<C, 8>(a, b, n, nl, ls, m, tw, inv); break;
			case 16: fft_pass<C, 16>(a, b, n, nl, ls, m, tw, inv); break;
			case 5: fft_pass<C, 5>(a, b, n, nl, ls, m, tw, inv); break;
			case 7: fft_pass<C, 7>(a, b, n, nl, ls, m, tw, inv); break;
			case 11: fft_pass<C, 11>(a, b, n, nl, ls, m, tw, inv); break;
			case 13: fft_pass<C, 13>(a, b, n, nl, ls, m, tw, inv); break;
			default: fft_pass_gen<C>(a, b, R, n, nl, ls, m, tw, inv); break;
		}
		__syncthreads();
		C *t = a;
		a = b;
		b = t;
		m *= R;
	}
	return a;
}

// ---------------------------------------------------------------------------------------------------------------
// Compile-time plans for power-of-two lengths. Every trip count, stride and divisor of a pass is a constant, so the
// element/line decomposition costs shifts instead of integer divisions and the passes unroll; the direction is a
// template parameter too. Radix MAXR first (16 for float, 8 for double), then the remaining power of two.

template <typename C, int R, int N, int NL, int LS, int M, int NT, bool INV>
__device__ __forceinline__ void fft_pass_s(const C *__restrict__ x, C *__restrict__ y, const C *__restrict__ tw)
{
	constexpr int NR = N / R, TOTAL = NR * NL, TSTEP = N / (M * R);
#pragma unroll 2
	for (int w = threadIdx.x; w < TOTAL; w += NT) {
		const int j = w / NL;
		const int l = w - j * NL;
		const int k = j & (M - 1);
		C v[R];
#pragma unroll
		for (int q = 0; q < R; q++) v[q] = x[(j + q * NR) * LS + l];
		if (M > 1) {
#pragma unroll
			for (int q = 1; q < R; q++) {
				C t = __ldg(tw + q * k * TSTEP);
				if (INV) t.y = -t.y;
				v[q] = cmul(v[q], t);
			}
		}
		dft<C, R>(v, INV, tw, N);
		const int base = (j - k) * R + k;
#pragma unroll
		for (int q = 0; q < R; q++) y[(base + q * M) * LS + l] = v[q];
	}
}

template <typename C, int N, int NL, int LS, int M, int MAXR, int NT, bool INV>
__device__ __forceinline__ C *fft_static(C *a, C *b, const C *__restrict__ tw)
{
	if constexpr (M >= N) {
		return a;
	}
	else {
		constexpr int REM = N / M;
		constexpr int R = REM >= MAXR ? MAXR : REM;
		fft_pass_s<C, R, N, NL, LS, M, NT, INV>(a, b, tw);
		__syncthreads();
		return fft_static<C, N, NL, LS, M * R, MAXR, NT, INV>(b, a, tw);
	}
}

// tile FFT with a compile-time plan when NS > 0 (power of two), the runtime plan otherwise
template <typename C, int NS, int NL, int LS, bool INV>
__device__ __forceinline__ C *tile_fft(C *a, C *b, const FftPlan &p, const C *__restrict__ tw)
{
	if constexpr (NS > 0) return fft_static<C, NS, NL, LS, 1, (sizeof(C) == 8 ? 16 : 8), 256, INV>(a, b, tw);
	else return fft_tile<C>(a, b, p, NL, LS, tw, INV);
}

// ---------------------------------------------------------------------------------------------------------------
// Asynchronous global -> shared copies of one complex element (cp.async, 8 or 16 bytes): the copy does not pass
// through registers, so a thread can have all of its tile loads in flight at once. With valid == false nothing is
// read and the destination is zero-filled (src-size 0); src must still be a mapped address.
template <typename C> __device__ __forceinline__ void cp_async_elem(C *dst, const C *src, bool valid)
{
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
	const int n = valid ? (int)sizeof(C) : 0;
	if (sizeof(C) == 16)
		asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
	else
		asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}
// bulk prefetch of bytes (a multiple of 16) at a 16-byte aligned global address into L2 (no completion to wait for)
__device__ __forceinline__ void prefetch_l2_bulk(const void *src, unsigned bytes)
{
	asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ---------------------------------------------------------------------------------------------------------------
// Register-resident two-step FFT of power-of-two length N = T*E for lines held by T consecutive lanes each
// (T <= E, T | 16): lane j1 of a line owns the E elements j1 + T*j2 in v[j2]. Step 1: DFT_E over j2 in registers,
// twiddle W_N^(j1*k2), transpose through the line's own shared buffer buf[k2*(T+1) + j1] (odd stride: conflict-free);
// step 2: each lane takes the E/T columns k2 = j1 + i*T and does DFT_T over j1 in registers. On return v[i*T + k1]
// holds X[j1 + i*T + E*k1], i.e. element j1 + T*(i + (E/T)*k1): the same "lane j1 owns j1 + T*j" form as the input,
// with j = i + (E/T)*k1 (reg_natural reorders it). Only the line's lanes synchronise (gmask = their warp lanes).
template <int N> struct RegShape {
	static constexpr int LOG = (N >= 512) ? 9 : (N >= 256) ? 8 : (N >= 128) ? 7 : (N >= 64) ? 6 : 5;
	static constexpr int T = 1 << (LOG / 2), E = N / T; // T <= E
	static constexpr int BUF = E * (T + 1);             // complex elements of a line's transpose buffer
};

// HALF_IN: the line's upper half is zero (v[j] for j >= E/2 is not read). twl: the step-1 twiddles lane-major,
// W_N^(j1*k2) at twl[k2*T + j1] (a line's T lanes read consecutive addresses).
template <typename C, int N, bool INV, bool HALF_IN = false>
__device__ __forceinline__ void reg_fft(C *v, C *buf, int j1, unsigned gmask, const C *__restrict__ twl)
{
	constexpr int T = RegShape<N>::T, E = RegShape<N>::E;
	if constexpr (HALF_IN) dft_half_in<C, E>(v, INV);
	else dft<C, E>(v, INV, twl, N);
#pragma unroll
	for (int k2 = 1; k2 < E; k2++) {
		C t = __ldg(twl + k2 * T + j1);
		if (INV) t.y = -t.y;
		v[k2] = cmul(v[k2], t);
	}
	__syncwarp(gmask);
#pragma unroll
	for (int k2 = 0; k2 < E; k2++) buf[k2 * (T + 1) + j1] = v[k2];
	__syncwarp(gmask);
#pragma unroll
	for (int i = 0; i < E / T; i++) {
		C u[T];
		const int k2 = j1 + i * T;
#pragma unroll
		for (int q = 0; q < T; q++) u[q] = buf[k2 * (T + 1) + q];
		dft<C, T>(u, INV, twl, N);
#pragma unroll
		for (int q = 0; q < T; q++) v[i * T + q] = u[q];
	}
}

// Line-fastest two-step FFT of NL lines by NT = NL*T threads: thread (l, j1) = (threadIdx % NL, threadIdx / NL)
// holds elements j1 + T*j of line l in v (j < E/2 with HALF_IN: the upper half is zero), so that consecutive threads
// hold consecutive lines and the caller's loads and stores along the lines' common contiguous axis coalesce. The
// step-1 results Y[j1][k2] go through xb laid out [k2][j1][l] (row groups of KS = T*NL + pad complex; with
// KS = NL mod 16 a warp's accesses of either phase fall on distinct bank pairs); one block barrier. On return
// v[i*T + k1] holds element (j1 + i*T) + E*k1 of line l. Every thread of the block must call it; the caller
// synchronises before reusing xb.
template <int NL, int T> __host__ __device__ constexpr int lf_ks() { return T * NL + (NL * (17 - T)) % 16; }
template <typename C, int N, int NL, bool INV, bool HALF_IN>
__device__ __forceinline__ void lf_fft(C *v, C *xb, int l, int j1, const C *__restrict__ tw)
{
	constexpr int T = RegShape<N>::T, E = RegShape<N>::E, KS = lf_ks<NL, T>();
	if constexpr (HALF_IN) dft_half_in<C, E>(v, INV);
	else dft<C, E>(v, INV, tw, N);
#pragma unroll
	for (int k2 = 1; k2 < E; k2++) {
		C t = __ldg(tw + j1 * k2);
		if (INV) t.y = -t.y;
		v[k2] = cmul(v[k2], t);
	}
#pragma unroll
	for (int k2 = 0; k2 < E; k2++) xb[k2 * KS + j1 * NL + l] = v[k2];
	__syncthreads();
#pragma unroll
	for (int i = 0; i < E / T; i++) {
		const int k2 = j1 + i * T;
		C u[T];
#pragma unroll
		for (int q = 0; q < T; q++) u[q] = xb[k2 * KS + q * NL + l];
		dft<C, T>(u, INV, tw, N);
#pragma unroll
		for (int k1 = 0; k1 < T; k1++) v[i * T + k1] = u[k1];
	}
}

// whether a kernel of compile-time length NS and arithmetic T transforms its lines with lf_fft (FP32, power-of-two
// 64..512) rather than with ping-pong Stockham passes over two tiles, and its thread count for NL lines
template <typename T, int NS> __host__ __device__ constexpr bool reg_cols() { return sizeof(T) == 4 && NS >= 64 && NS <= 512; }
template <typename T, int NS, int NL> __host__ __device__ constexpr int col_threads()
{
	return reg_cols<T, NS>() ? NL * RegShape<NS>::T : 256;
}
// resident blocks per SM the column kernels are compiled for (at most 56 registers a thread up to length 256)
template <typename T, int NS, int NL> __host__ __device__ constexpr int col_minblocks()
{
	return (reg_cols<T, NS>() && NS <= 256) ? 65536 / (col_threads<T, NS, NL>() * 56) : 1;
}

// reorder the output of reg_fft into the input form (v[j] = element j1 + T*j)
template <typename C, int N> __device__ __forceinline__ void reg_natural(C *v)
{
	constexpr int T = RegShape<N>::T, E = RegShape<N>::E;
	if constexpr (E != T) {
		C w[E];
#pragma unroll
		for (int i = 0; i < E / T; i++)
#pragma unroll
			for (int k1 = 0; k1 < T; k1++) w[i + (E / T) * k1] = v[i * T + k1];
#pragma unroll
		for (int j = 0; j < E; j++) v[j] = w[j];
	}
}

} // namespace adda
