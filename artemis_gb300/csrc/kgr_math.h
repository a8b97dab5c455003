/*
 * kgr_math.h -- deterministic float arithmetic shared by host and device.
 *
 * Every function here is written with an explicit evaluation order and uses
 * only IEEE-754 correctly rounded operations (+ - * / sqrt floor).  Compiled
 * with FMA contraction disabled (nvcc -fmad=false, g++ -ffp-contract=off) and
 * without flush-to-zero, the same source produces bit-identical results on
 * the GPU (sm_103a) and on any IEEE host (x86-64 or aarch64).  That is what
 * makes hit IDs, bounce directions and radiance comparable bit for bit
 * between the CUDA kernels and the CPU oracle.
 *
 * Vector helpers follow the operator definitions of the reference's
 * include/cuda/math.cuh (float3 ops :393-541, normalize :526, fract :2604,
 * rotate :2653): e.g. `v / s` is `v * (1.0f / s)`, `normalize(v)` is
 * `v * (1.0f / sqrtf(dot(v, v)))`, `dot` sums left to right.
 *
 * The transcendental functions (sin, cos, tan, atan, acos) are this
 * project's own: Cody-Waite reduction by pi/2 (three-part split computed
 * from pi to 200 bits) followed by Taylor polynomials on |r| <= pi/4
 * (sin/cos) or |r| <= tan(pi/12) (atan).  Their error is within a couple of
 * ulp of the true value, which is the same accuracy class as the fast
 * intrinsics (__tanf, __cosf, __sinf) the reference calls in
 * include/cuda/brdf.cuh:188,217-218,408-428.
 */
#ifndef KGR_MATH_H_
#define KGR_MATH_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define KGR_HD __host__ __device__ __forceinline__
#else
#define KGR_HD inline
#endif

#if !defined(__CUDA_ARCH__)
#include <math.h>
#include <string.h>
#endif

namespace kgr {

/* ---------------------------------------------------------------- bits -- */

KGR_HD uint32_t f2u(float f)
{
#if defined(__CUDA_ARCH__)
	return __float_as_uint(f);
#else
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
#endif
}

KGR_HD float u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
	return __uint_as_float(u);
#else
	float f;
	memcpy(&f, &u, 4);
	return f;
#endif
}

KGR_HD float ksqrt(float x)
{
#if defined(__CUDA_ARCH__)
	return __fsqrt_rn(x);
#else
	return sqrtf(x);
#endif
}

KGR_HD float kfloor(float x) { return floorf(x); }
KGR_HD float kabs(float x) { return fabsf(x); }
KGR_HD float kmax(float a, float b) { return fmaxf(a, b); }
KGR_HD float kmin(float a, float b) { return fminf(a, b); }
KGR_HD bool kisnan(float x) { return x != x; }

/* -------------------------------------------------------------- float3 -- */

struct f3 {
	float x, y, z;
};

KGR_HD f3 mk(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
KGR_HD f3 mk(float s) { return mk(s, s, s); }

KGR_HD f3 operator-(const f3 &a) { return mk(-a.x, -a.y, -a.z); }
KGR_HD f3 operator+(const f3 &a, const f3 &b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
KGR_HD f3 operator-(const f3 &a, const f3 &b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
KGR_HD f3 operator*(const f3 &a, const f3 &b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
KGR_HD f3 operator*(const f3 &a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
KGR_HD f3 operator*(float s, const f3 &a) { return mk(a.x * s, a.y * s, a.z * s); }
KGR_HD f3 operator-(float s, const f3 &a) { return mk(s - a.x, s - a.y, s - a.z); }
KGR_HD f3 operator-(const f3 &a, float s) { return mk(a.x - s, a.y - s, a.z - s); }
/* math.cuh:464-468: division by a scalar multiplies by its reciprocal */
KGR_HD f3 operator/(const f3 &a, float s) { float inv = 1.0f / s; return a * inv; }
KGR_HD void operator+=(f3 &a, const f3 &b) { a = a + b; }
KGR_HD void operator*=(f3 &a, const f3 &b) { a = a * b; }
KGR_HD void operator*=(f3 &a, float s) { a = a * s; }
KGR_HD void operator/=(f3 &a, float s) { a = a / s; }

KGR_HD float dot(const f3 &a, const f3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KGR_HD f3 cross(const f3 &a, const f3 &b)
{
	return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
KGR_HD float length(const f3 &v) { return ksqrt(dot(v, v)); }
KGR_HD f3 normalize(const f3 &v) { float inv = 1.0f / ksqrt(dot(v, v)); return v * inv; }
/* math.cuh:539-542 */
KGR_HD f3 reflect(const f3 &i, const f3 &n) { return i - 2.0f * n * dot(n, i); }
KGR_HD f3 fmin3(const f3 &a, const f3 &b) { return mk(kmin(a.x, b.x), kmin(a.y, b.y), kmin(a.z, b.z)); }
KGR_HD f3 fmax3(const f3 &a, const f3 &b) { return mk(kmax(a.x, b.x), kmax(a.y, b.y), kmax(a.z, b.z)); }
KGR_HD float comp(const f3 &v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
KGR_HD bool anynan(const f3 &v) { return kisnan(v.x) || kisnan(v.y) || kisnan(v.z); }

/* math.cuh:2604-2607 */
KGR_HD float fract(float x) { return x - kfloor(x); }
KGR_HD f3 fract(const f3 &v) { return mk(fract(v.x), fract(v.y), fract(v.z)); }

/* ------------------------------------------------------ transcendentals -- */

/* pi/2 = PIO2_HI + PIO2_MID + PIO2_LO; HI and MID carry 12 significant bits
 * so k * HI and k * MID are exact for |k| < 2^12. */
#define KGR_PIO2_HI 1.5703125f
#define KGR_PIO2_MID 4.837512970e-04f
#define KGR_PIO2_LO 7.549790126e-08f
#define KGR_2_OVER_PI 0.636619747f
#define KGR_PI_F 3.14159265358979323846f
#define KGR_PIO2_F 1.57079637f
#define KGR_PIO6_F 0.523598790f
#define KGR_SQRT3_F 1.73205078f
#define KGR_TAN_PI12_F 0.267949194f

/* sin and cos of r for |r| <= pi/4 (Taylor series, truncation < 1e-9). */
KGR_HD float sin_kernel(float r)
{
	float z = r * r;
	float p = 2.75573192e-06f;                 /*  1/9! */
	p = -1.98412698e-04f + z * p;              /* -1/7! */
	p = 8.33333333e-03f + z * p;               /*  1/5! */
	p = -1.66666667e-01f + z * p;              /* -1/3! */
	return r + (r * z) * p;
}

KGR_HD float cos_kernel(float r)
{
	float z = r * r;
	float p = -2.75573192e-07f;                /* -1/10! */
	p = 2.48015873e-05f + z * p;               /*  1/8!  */
	p = -1.38888889e-03f + z * p;              /* -1/6!  */
	p = 4.16666667e-02f + z * p;               /*  1/4!  */
	return (1.0f - 0.5f * z) + (z * z) * p;
}

/* Reduce x to r in [-pi/4, pi/4] and quadrant q (mod 4). */
KGR_HD float reduce_pio2(float x, int &q)
{
	float k = kfloor(x * KGR_2_OVER_PI + 0.5f);
	float r = ((x - k * KGR_PIO2_HI) - k * KGR_PIO2_MID) - k * KGR_PIO2_LO;
	q = ((int)k) & 3;
	return r;
}

KGR_HD void ksincos(float x, float &s, float &c)
{
	int q;
	float r = reduce_pio2(x, q);
	float sr = sin_kernel(r), cr = cos_kernel(r);
	switch (q) {
	case 0: s = sr; c = cr; break;
	case 1: s = cr; c = -sr; break;
	case 2: s = -sr; c = -cr; break;
	default: s = -cr; c = sr; break;
	}
}

KGR_HD float ksin(float x) { float s, c; ksincos(x, s, c); return s; }
KGR_HD float kcos(float x) { float s, c; ksincos(x, s, c); return c; }
KGR_HD float ktan(float x) { float s, c; ksincos(x, s, c); return s / c; }

/* atan for |y| <= tan(pi/12) (Taylor series, truncation < 2e-9). */
KGR_HD float atan_kernel(float y)
{
	float z = y * y;
	float p = 7.69230769e-02f;                 /*  1/13 */
	p = -9.09090909e-02f + z * p;              /* -1/11 */
	p = 1.11111111e-01f + z * p;               /*  1/9  */
	p = -1.42857143e-01f + z * p;              /* -1/7  */
	p = 2.00000000e-01f + z * p;               /*  1/5  */
	p = -3.33333333e-01f + z * p;              /* -1/3  */
	return y + (y * z) * p;
}

KGR_HD float katan(float x)
{
	if (kisnan(x))
		return x;
	bool neg = x < 0.0f;
	float a = neg ? -x : x;
	bool inv = a > 1.0f;
	if (inv)
		a = 1.0f / a;
	float r;
	if (a > KGR_TAN_PI12_F)
		r = KGR_PIO6_F + atan_kernel((a * KGR_SQRT3_F - 1.0f) / (a + KGR_SQRT3_F));
	else
		r = atan_kernel(a);
	if (inv)
		r = KGR_PIO2_F - r;
	return neg ? -r : r;
}

/* acos(x) = 2 atan(sqrt((1 - x) / (1 + x))) on [-1, 1]; NaN outside. */
KGR_HD float kacos(float x)
{
	if (!(x >= -1.0f && x <= 1.0f))
		return (x - x) / (x - x);
	return 2.0f * katan(ksqrt((1.0f - x) / (1.0f + x)));
}

/* atan2(y, x): katan(y / x) moved to the quadrant of (x, y); +-pi/2 on the
 * y axis and 0 at the origin. */
KGR_HD float katan2(float y, float x)
{
	if (kisnan(x) || kisnan(y))
		return x + y;
	if (x == 0.0f)
		return y > 0.0f ? KGR_PIO2_F : (y < 0.0f ? -KGR_PIO2_F : 0.0f);
	float r = katan(y / x);
	if (x < 0.0f)
		r = y < 0.0f ? r - KGR_PI_F : r + KGR_PI_F;
	return r;
}

/* asin(x) = atan(x / sqrt(1 - x^2)) on (-1, 1), +-pi/2 at +-1; NaN outside. */
KGR_HD float kasin(float x)
{
	if (!(x >= -1.0f && x <= 1.0f))
		return (x - x) / (x - x);
	if (x == 1.0f || x == -1.0f)
		return x * KGR_PIO2_F;
	return katan(x / ksqrt((1.0f - x) * (1.0f + x)));
}

/* powf(x, 2|4|5) for the three integer exponents brdf.cuh uses. */
KGR_HD float kpow2(float x) { return x * x; }
KGR_HD float kpow4(float x) { float x2 = x * x; return x2 * x2; }
KGR_HD float kpow5(float x) { float x2 = x * x; return (x2 * x2) * x; }

KGR_HD float clampf(float f, float a, float b) { return kmax(a, kmin(f, b)); }

/* ------------------------------------------------------------------ RNG -- */

/* pcg3d hash over the bit pattern of a float3 seed (random.cuh:14-26). */
KGR_HD void pcg3d(uint32_t &x, uint32_t &y, uint32_t &z)
{
	x = x * 1664525u + 1013904223u;
	y = y * 1664525u + 1013904223u;
	z = z * 1664525u + 1013904223u;
	x += y * z;
	y += z * x;
	z += x * y;
	x ^= x >> 16u;
	y ^= y >> 16u;
	z ^= z >> 16u;
	x += y * z;
	y += z * x;
	z += x * y;
}

/* pcg3f (random.cuh:28-38): hash the seed, map the mantissas into [1,2),
 * subtract one; the seed is replaced by the result, which is returned. */
KGR_HD f3 pcg3f(f3 &seed)
{
	uint32_t x = f2u(seed.x), y = f2u(seed.y), z = f2u(seed.z);
	pcg3d(x, y, z);
	x = (x & 0x007fffffu) | 0x3f800000u;
	y = (y & 0x007fffffu) | 0x3f800000u;
	z = (z & 0x007fffffu) | 0x3f800000u;
	seed = mk(u2f(x) - 1.0f, u2f(y) - 1.0f, u2f(z) - 1.0f);
	return seed;
}

/* rand_uniform (random.cuh:40-44) */
KGR_HD float rand_uniform(f3 &seed)
{
	seed = pcg3f(seed);
	return fract(seed.x);
}

/* rand_uniform(lim) (random.cuh:46-50) */
KGR_HD unsigned int rand_uniform(unsigned int lim, f3 &seed)
{
	return (unsigned int)(rand_uniform(seed) * lim);
}

/* rand_uniform_3f (random.cuh:52-57) */
KGR_HD f3 rand_uniform_3f(f3 &seed)
{
	seed = pcg3f(seed);
	return fract(seed);
}

/* Per-pixel stream: seed bits {pixel ^ stream, pixel, stream}.  `stream` is
 * the frame index times samples-per-frame plus the sample index; salt
 * separates independent streams of one pixel (0 for paths). */
KGR_HD f3 pixel_seed(uint32_t pixel, uint32_t stream, uint32_t salt)
{
	return mk(u2f(pixel ^ stream), u2f(pixel ^ salt), u2f(stream));
}

/* ------------------------------------------------- GI reservoir packing -- */

/* A unit normal in octahedral form, 12 bits per coordinate, and a sample
 * count M clamped to 255, in one 32-bit word: bits 0-11 u, 12-23 v, 24-31 M.
 * Only exact operations, so both sides pack and unpack identically. */
KGR_HD uint32_t pack_normal_m(const f3 &n, int32_t m)
{
	float s = kabs(n.x) + kabs(n.y) + kabs(n.z);
	float px = n.x / s, py = n.y / s;
	if (n.z < 0.0f) {
		float qx = (1.0f - kabs(py)) * (px >= 0.0f ? 1.0f : -1.0f);
		float qy = (1.0f - kabs(px)) * (py >= 0.0f ? 1.0f : -1.0f);
		px = qx;
		py = qy;
	}
	px = clampf(px, -1.0f, 1.0f);
	py = clampf(py, -1.0f, 1.0f);
	uint32_t u = (uint32_t)(int32_t)kfloor(px * 2047.0f + 2047.5f);
	uint32_t v = (uint32_t)(int32_t)kfloor(py * 2047.0f + 2047.5f);
	uint32_t mm = (uint32_t)(m < 0 ? 0 : (m > 255 ? 255 : m));
	return (u & 0xfffu) | ((v & 0xfffu) << 12) | (mm << 24);
}

KGR_HD f3 unpack_normal(uint32_t w)
{
	float px = ((float)(int32_t)(w & 0xfffu) - 2047.0f) / 2047.0f;
	float py = ((float)(int32_t)((w >> 12) & 0xfffu) - 2047.0f) / 2047.0f;
	float pz = 1.0f - kabs(px) - kabs(py);
	if (pz < 0.0f) {
		float qx = (1.0f - kabs(py)) * (px >= 0.0f ? 1.0f : -1.0f);
		float qy = (1.0f - kabs(px)) * (py >= 0.0f ? 1.0f : -1.0f);
		px = qx;
		py = qy;
	}
	return normalize(mk(px, py, pz));
}

KGR_HD int32_t unpack_m(uint32_t w) { return (int32_t)(w >> 24); }

KGR_HD float max3(const f3 &v) { return kmax(v.x, kmax(v.y, v.z)); }

/* rotate (math.cuh:2653-2668): express s in a frame around n. */
KGR_HD f3 rotate(const f3 &s, const f3 &n)
{
	f3 w = n;
	f3 a = mk(0.0f, 1.0f, 0.0f);
	if (kabs(dot(w, a)) > 0.999f)
		a = mk(0.0f, 0.0f, 1.0f);
	f3 u = normalize(cross(w, a));
	f3 v = normalize(cross(w, u));
	return u * s.x + v * s.y + w * s.z;
}

} /* namespace kgr */

#endif
