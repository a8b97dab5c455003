/*
 * ref_math.h -- the oracle's own float arithmetic (TEST INFRASTRUCTURE).
 *
 * Written separately from the product's kernels so that a slip in either
 * side's helpers shows up as a parity failure instead of passing on both.
 * Only IEEE-754 correctly rounded operations, each expression in a fixed
 * order; compiled with -ffp-contract=off.
 *
 *  - float3 helpers: the operators of the reference's include/cuda/math.cuh
 *    (:393-541; a scalar division is a multiplication by the reciprocal,
 *    :464-468; normalize multiplies by 1 / sqrt(dot), :526; fract, :2604;
 *    rotate, :2653-2668).
 *  - RNG: pcg3d / pcg3f / rand_uniform / rand_uniform_3f of
 *    include/cuda/random.cuh:14-58 (pinned by the known-answer vectors the
 *    reference's own header produces, tests/golden/reference_kat.json).
 *  - sin, cos, tan, atan, acos, asin, atan2: the project's specification of
 *    the reference's fast intrinsics (__sinf, __cosf, __tanf in
 *    include/cuda/brdf.cuh): a three-part Cody-Waite reduction by pi/2 and
 *    Taylor polynomials of degree 9/10 (sin/cos) and 13 (atan, with the
 *    pi/6 argument shift above tan(pi/12)); checked against float64 in
 *    tests/test_oracle_kat.py.
 *  - the 32-bit octahedral normal + sample-count word of the GI reservoirs.
 */
#ifndef KGR_ORACLE_REF_MATH_H_
#define KGR_ORACLE_REF_MATH_H_

#include <math.h>
#include <stdint.h>
#include <string.h>

namespace oref {

inline uint32_t f2u(float f)
{
	uint32_t u;
	memcpy(&u, &f, sizeof u);
	return u;
}

inline float u2f(uint32_t u)
{
	float f;
	memcpy(&f, &u, sizeof f);
	return f;
}

inline float ksqrt(float x) { return sqrtf(x); }
inline float kfloor(float x) { return floorf(x); }
inline float kabs(float x) { return fabsf(x); }
inline float kmax(float a, float b) { return fmaxf(a, b); }
inline float kmin(float a, float b) { return fminf(a, b); }
inline bool kisnan(float x) { return !(x == x); }

/* ------------------------------------------------------------- float3 -- */

struct f3 {
	float x, y, z;
};

inline f3 mk(float x, float y, float z)
{
	f3 v = {x, y, z};
	return v;
}
inline f3 mk(float s) { return mk(s, s, s); }

inline f3 operator-(const f3 &a) { return mk(-a.x, -a.y, -a.z); }
inline f3 operator+(const f3 &a, const f3 &b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline f3 operator-(const f3 &a, const f3 &b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline f3 operator*(const f3 &a, const f3 &b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline f3 operator*(const f3 &a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline f3 operator*(float s, const f3 &a) { return a * s; }
inline f3 operator-(float s, const f3 &a) { return mk(s - a.x, s - a.y, s - a.z); }
inline f3 operator-(const f3 &a, float s) { return mk(a.x - s, a.y - s, a.z - s); }
inline f3 operator/(const f3 &a, float s)
{
	float r = 1.0f / s;
	return a * r;
}
inline void operator+=(f3 &a, const f3 &b) { a = a + b; }
inline void operator*=(f3 &a, const f3 &b) { a = a * b; }
inline void operator*=(f3 &a, float s) { a = a * s; }
inline void operator/=(f3 &a, float s) { a = a / s; }

inline float dot(const f3 &a, const f3 &b)
{
	float s = a.x * b.x;
	s = s + a.y * b.y;
	return s + a.z * b.z;
}
inline f3 cross(const f3 &a, const f3 &b)
{
	float x = a.y * b.z - a.z * b.y;
	float y = a.z * b.x - a.x * b.z;
	float z = a.x * b.y - a.y * b.x;
	return mk(x, y, z);
}
inline float length(const f3 &v) { return ksqrt(dot(v, v)); }
inline f3 normalize(const f3 &v)
{
	float r = 1.0f / ksqrt(dot(v, v));
	return v * r;
}
inline f3 reflect(const f3 &i, const f3 &n) { return i - 2.0f * n * dot(n, i); }
inline f3 fmin3(const f3 &a, const f3 &b) { return mk(kmin(a.x, b.x), kmin(a.y, b.y), kmin(a.z, b.z)); }
inline f3 fmax3(const f3 &a, const f3 &b) { return mk(kmax(a.x, b.x), kmax(a.y, b.y), kmax(a.z, b.z)); }
inline float comp(const f3 &v, int i)
{
	const float c[3] = {v.x, v.y, v.z};
	return c[i];
}
inline bool anynan(const f3 &v) { return kisnan(v.x) || kisnan(v.y) || kisnan(v.z); }
inline float fract(float x) { return x - kfloor(x); }
inline f3 fract(const f3 &v) { return mk(fract(v.x), fract(v.y), fract(v.z)); }
inline float max3(const f3 &v) { return kmax(v.x, kmax(v.y, v.z)); }
inline float clampf(float f, float lo, float hi) { return kmax(lo, kmin(f, hi)); }

/* ------------------------------------------------------ transcendental -- */

/* pi/2 split in three: the first two parts have 12 significant bits, so
 * their products with a quadrant count below 2^12 are exact. */
const float PIO2_A = 1.5703125f;
const float PIO2_B = 4.837512970e-04f;
const float PIO2_C = 7.549790126e-08f;
const float TWO_OVER_PI = 0.636619747f;
const float PI_F = 3.14159265358979323846f;
const float HALF_PI_F = 1.57079637f;
const float SIXTH_PI_F = 0.523598790f;
const float SQRT3_F = 1.73205078f;
const float TAN_PI12_F = 0.267949194f;

/* Horner evaluation over z = r^2, highest coefficient first */
inline float horner(float z, const float *c, int n)
{
	float p = c[0];
	for (int i = 1; i < n; i++)
		p = c[i] + z * p;
	return p;
}

/* sin r = r + r^3 (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 / 9!))) */
inline float sin_poly(float r)
{
	static const float c[4] = {2.75573192e-06f, -1.98412698e-04f, 8.33333333e-03f, -1.66666667e-01f};
	float z = r * r;
	return r + (r * z) * horner(z, c, 4);
}

/* cos r = (1 - r^2/2) + r^4 (1/4! + r^2 (-1/6! + r^2 (1/8! - r^2/10!))) */
inline float cos_poly(float r)
{
	static const float c[4] = {-2.75573192e-07f, 2.48015873e-05f, -1.38888889e-03f, 4.16666667e-02f};
	float z = r * r;
	return (1.0f - 0.5f * z) + (z * z) * horner(z, c, 4);
}

inline void ksincos(float x, float &s, float &c)
{
	float k = kfloor(x * TWO_OVER_PI + 0.5f);
	float r = x - k * PIO2_A;
	r = r - k * PIO2_B;
	r = r - k * PIO2_C;
	float sr = sin_poly(r), cr = cos_poly(r);
	int q = ((int)k) & 3;
	if (q == 0) {
		s = sr;
		c = cr;
	} else if (q == 1) {
		s = cr;
		c = -sr;
	} else if (q == 2) {
		s = -sr;
		c = -cr;
	} else {
		s = -cr;
		c = sr;
	}
}

inline float ksin(float x)
{
	float s, c;
	ksincos(x, s, c);
	return s;
}
inline float kcos(float x)
{
	float s, c;
	ksincos(x, s, c);
	return c;
}
inline float ktan(float x)
{
	float s, c;
	ksincos(x, s, c);
	return s / c;
}

/* atan y = y + y^3 (-1/3 + y^2 (1/5 + ... + y^2 / 13)) for |y| <= tan(pi/12) */
inline float atan_poly(float y)
{
	static const float c[6] = {7.69230769e-02f, -9.09090909e-02f, 1.11111111e-01f, -1.42857143e-01f,
		2.00000000e-01f, -3.33333333e-01f};
	float z = y * y;
	return y + (y * z) * horner(z, c, 6);
}

inline float katan(float x)
{
	if (kisnan(x))
		return x;
	float a = x < 0.0f ? -x : x;
	bool big = a > 1.0f;
	if (big)
		a = 1.0f / a;
	/* above tan(pi/12): atan a = pi/6 + atan((a sqrt3 - 1) / (a + sqrt3)) */
	float r = a > TAN_PI12_F ? SIXTH_PI_F + atan_poly((a * SQRT3_F - 1.0f) / (a + SQRT3_F)) : atan_poly(a);
	if (big)
		r = HALF_PI_F - r;
	return x < 0.0f ? -r : r;
}

inline float nan_of(float x) { return (x - x) / (x - x); }

inline float kacos(float x)
{
	if (!(x >= -1.0f && x <= 1.0f))
		return nan_of(x);
	return 2.0f * katan(ksqrt((1.0f - x) / (1.0f + x)));
}

inline float katan2(float y, float x)
{
	if (kisnan(x) || kisnan(y))
		return x + y;
	if (x == 0.0f) {
		if (y > 0.0f)
			return HALF_PI_F;
		return y < 0.0f ? -HALF_PI_F : 0.0f;
	}
	float r = katan(y / x);
	if (x < 0.0f)
		r = y < 0.0f ? r - PI_F : r + PI_F;
	return r;
}

inline float kasin(float x)
{
	if (!(x >= -1.0f && x <= 1.0f))
		return nan_of(x);
	if (x == 1.0f || x == -1.0f)
		return x * HALF_PI_F;
	return katan(x / ksqrt((1.0f - x) * (1.0f + x)));
}

inline float kpow2(float x) { return x * x; }
inline float kpow4(float x)
{
	float x2 = x * x;
	return x2 * x2;
}
inline float kpow5(float x)
{
	float x2 = x * x;
	return (x2 * x2) * x;
}

/* ---------------------------------------------------------------- RNG -- */

/* pcg3d (random.cuh:14-26): an LCG step per lane, then two rounds of
 * cross-lane mixing around a 16-bit xorshift */
inline void pcg3d(uint32_t &x, uint32_t &y, uint32_t &z)
{
	const uint32_t mul = 1664525u, inc = 1013904223u;
	x = x * mul + inc;
	y = y * mul + inc;
	z = z * mul + inc;
	for (int round = 0; round < 2; round++) {
		x += y * z;
		y += z * x;
		z += x * y;
		if (round == 0) {
			x ^= x >> 16u;
			y ^= y >> 16u;
			z ^= z >> 16u;
		}
	}
}

/* pcg3f (random.cuh:28-38): the hashed bits as mantissas in [1, 2), minus
 * one; the seed becomes the result */
inline f3 pcg3f(f3 &seed)
{
	uint32_t b[3] = {f2u(seed.x), f2u(seed.y), f2u(seed.z)};
	pcg3d(b[0], b[1], b[2]);
	float v[3];
	for (int i = 0; i < 3; i++)
		v[i] = u2f((b[i] & 0x007fffffu) | 0x3f800000u) - 1.0f;
	seed = mk(v[0], v[1], v[2]);
	return seed;
}

inline float rand_uniform(f3 &seed)
{
	seed = pcg3f(seed);
	return fract(seed.x);
}

inline unsigned int rand_uniform(unsigned int lim, f3 &seed) { return (unsigned int)(rand_uniform(seed) * lim); }

inline f3 rand_uniform_3f(f3 &seed)
{
	seed = pcg3f(seed);
	return fract(seed);
}

/* the per-pixel stream: bits {pixel ^ stream, pixel ^ salt, stream} */
inline f3 pixel_seed(uint32_t pixel, uint32_t stream, uint32_t salt)
{
	return mk(u2f(pixel ^ stream), u2f(pixel ^ salt), u2f(stream));
}

/* -------------------------------------------------- GI reservoir word -- */

/* octahedral fold of the lower hemisphere */
inline void oct_fold(float &px, float &py)
{
	float sx = px >= 0.0f ? 1.0f : -1.0f, sy = py >= 0.0f ? 1.0f : -1.0f;
	float qx = (1.0f - kabs(py)) * sx;
	float qy = (1.0f - kabs(px)) * sy;
	px = qx;
	py = qy;
}

/* bits 0-11 u, 12-23 v of the octahedral normal, 24-31 M (clamped to 255) */
inline uint32_t pack_normal_m(const f3 &n, int32_t m)
{
	float s = kabs(n.x) + kabs(n.y) + kabs(n.z);
	float px = n.x / s, py = n.y / s;
	if (n.z < 0.0f)
		oct_fold(px, py);
	px = clampf(px, -1.0f, 1.0f);
	py = clampf(py, -1.0f, 1.0f);
	uint32_t u = (uint32_t)(int32_t)kfloor(px * 2047.0f + 2047.5f);
	uint32_t v = (uint32_t)(int32_t)kfloor(py * 2047.0f + 2047.5f);
	uint32_t mm = m < 0 ? 0u : (m > 255 ? 255u : (uint32_t)m);
	return (u & 0xfffu) | ((v & 0xfffu) << 12) | (mm << 24);
}

inline f3 unpack_normal(uint32_t w)
{
	float px = ((float)(int32_t)(w & 0xfffu) - 2047.0f) / 2047.0f;
	float py = ((float)(int32_t)((w >> 12) & 0xfffu) - 2047.0f) / 2047.0f;
	float pz = 1.0f - kabs(px) - kabs(py);
	if (pz < 0.0f)
		oct_fold(px, py);
	return normalize(mk(px, py, pz));
}

inline int32_t unpack_m(uint32_t w) { return (int32_t)(w >> 24); }

/* rotate (math.cuh:2653-2668): s in the frame {u, v, n} around n */
inline f3 rotate(const f3 &s, const f3 &n)
{
	f3 a = kabs(dot(n, mk(0.0f, 1.0f, 0.0f))) > 0.999f ? mk(0.0f, 0.0f, 1.0f) : mk(0.0f, 1.0f, 0.0f);
	f3 u = normalize(cross(n, a));
	f3 v = normalize(cross(n, u));
	return u * s.x + v * s.y + n * s.z;
}

} /* namespace oref */

#endif
