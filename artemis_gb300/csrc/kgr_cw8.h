/*
 * kgr_cw8.h -- quantisation of the compressed eight-child nodes (CwNode),
 * shared by the host builder (bvh_build.cpp) and the device refit
 * (refit.cu) so both write the same bytes for the same boxes.
 *
 * A node's grid on each axis is p + q * 2^e for q = 0..255.  e is the
 * smallest exponent with 2^e >= extent / 253, raised until the children's
 * boxes fit; p sits at least one grid step below the lowest child plane
 * (rounded down to a float).  Each child plane is then moved outward to the
 * grid by at least half a step: lo = floor((plane - p) / 2^e - 1/2), hi =
 * ceil((plane - p) / 2^e + 1/2), so p + q 2^e encloses the padded box in
 * exact arithmetic with room to spare.  Everything is IEEE double
 * arithmetic without contraction (frexp, ldexp, floor and ceil are exact),
 * so host and device agree bit for bit.
 */
#ifndef KGR_CW8_H_
#define KGR_CW8_H_

#include <math.h>
#include <stdint.h>

#include <cuda_runtime.h>

#include "kgr_math.h"

namespace kgr {

/* largest float <= x */
KGR_HD float cw_float_down(double x)
{
	float f = (float)x;
	if ((double)f > x)
		f = nextafterf(f, -INFINITY);
	return f;
}

/* Grid of one axis for planes spanning [lo, hi]: the exponent (unbiased)
 * and the origin. */
KGR_HD void cw_axis_grid(float lo, float hi, int &e, float &p)
{
	double ext = (double)hi - (double)lo;
	int k = -126;
	if (ext > 0.0) {
		int x = 0;
		double m = frexp(ext / 253.0, &x); /* ext / 253 = m 2^x, m in [0.5, 1) */
		k = (m == 0.5) ? x - 1 : x;
	}
	if (k < -126)
		k = -126;
	for (; k < 127; k++) {
		double s = ldexp(1.0, k);
		p = cw_float_down((double)lo - s);
		if (((double)hi - (double)p) / s + 0.5 <= 255.0)
			break;
	}
	if (k >= 127) { /* cannot happen for finite boxes of float coordinates */
		k = 127;
		p = cw_float_down((double)lo - ldexp(1.0, k));
	}
	e = k;
}

KGR_HD uint32_t cw_qlo(float plane, float p, double s)
{
	double q = floor(((double)plane - (double)p) / s - 0.5);
	return (uint32_t)(q < 0.0 ? 0.0 : (q > 255.0 ? 255.0 : q));
}

KGR_HD uint32_t cw_qhi(float plane, float p, double s)
{
	double q = ceil(((double)plane - (double)p) / s + 0.5);
	return (uint32_t)(q < 0.0 ? 0.0 : (q > 255.0 ? 255.0 : q));
}

/* Fill origin (p, exponents, imask) and the three quantised plane words of
 * a node from its children's padded boxes.  used: bit j set when slot j
 * holds a child (internal or leaf); lo/hi: 8 x 3 floats.  Empty slots get
 * lo = 255, hi = 0 (the walk skips them by their slot mask anyway). */
KGR_HD void cw_quantize(const float lo[8][3], const float hi[8][3], uint32_t used, uint32_t imask, float4 &origin,
		uint4 &qa, uint4 &qb, uint4 &qc)
{
	float pl[3], ph[3];
	for (int a = 0; a < 3; a++) {
		pl[a] = INFINITY;
		ph[a] = -INFINITY;
	}
	for (int j = 0; j < 8; j++) {
		if (!(used >> j & 1u))
			continue;
		for (int a = 0; a < 3; a++) {
			pl[a] = lo[j][a] < pl[a] ? lo[j][a] : pl[a];
			ph[a] = hi[j][a] > ph[a] ? hi[j][a] : ph[a];
		}
	}
	int e[3];
	float p[3];
	for (int a = 0; a < 3; a++) {
		if (!used) {
			pl[a] = 0.0f;
			ph[a] = 0.0f;
		}
		cw_axis_grid(pl[a], ph[a], e[a], p[a]);
	}
	uint32_t words[12] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
	/* word order: lo.x lo.x lo.y lo.y | lo.z lo.z hi.x hi.x | hi.y hi.y hi.z hi.z */
	for (int j = 0; j < 8; j++) {
		bool u = (used >> j & 1u) != 0;
		for (int a = 0; a < 3; a++) {
			double s = ldexp(1.0, e[a]);
			uint32_t ql = u ? cw_qlo(lo[j][a], p[a], s) : 255u;
			uint32_t qh = u ? cw_qhi(hi[j][a], p[a], s) : 0u;
			int wl = 2 * a + (j >> 2), wh = 6 + 2 * a + (j >> 2);
			words[wl] |= ql << (8 * (j & 3));
			words[wh] |= qh << (8 * (j & 3));
		}
	}
	uint32_t ebits = (uint32_t)(e[0] + 127) | (uint32_t)(e[1] + 127) << 8 | (uint32_t)(e[2] + 127) << 16
		| (imask & 0xffu) << 24;
	origin = make_float4(p[0], p[1], p[2], u2f(ebits));
	qa = make_uint4(words[0], words[1], words[2], words[3]);
	qb = make_uint4(words[4], words[5], words[6], words[7]);
	qc = make_uint4(words[8], words[9], words[10], words[11]);
}

} /* namespace kgr */

#endif
