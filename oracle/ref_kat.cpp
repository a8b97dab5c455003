/*
 * ref_kat.cpp -- known-answer vectors from the reference's own headers.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) against
 * the reference sources where they lie (REFERENCE=<path to the artemis
 * checkout>), into oracle/_ref/ref_kat.  It includes, unmodified:
 *   include/cuda/random.cuh   pcg3d, pcg3f, rand_uniform, rand_uniform_3f
 *   include/cuda/math.cuh     float3 operators, normalize, rotate, fract
 *   include/cuda/brdf.cuh     GGX brdf/pdf/sample/eval
 *   include/optix/lighting.cuh intersects_triangle, TriangleLight,
 *                             sample_area_light
 * Host compilation needs three shims, stated here: `__device__` and
 * `__forceinline__` expand to nothing/inline, the fast intrinsics
 * __tanf/__cosf/__sinf map to the C library's tanf/cosf/sinf, and a float
 * overload of min() (Glass::sample calls min(float, float), which the
 * reference only gets from the CUDA device headers).  The program prints
 * JSON on stdout; tests/golden/gen_golden.py stores it as fixtures.
 */
#include <cmath>
#include <cstdio>
#include <cstdint>
using std::abs;
using std::fmax;
using std::fmaxf;
using std::fminf;
using std::sqrt;
#define __forceinline__ inline
#define __device__
#define __tanf tanf
#define __cosf cosf
#define __sinf sinf
#include "include/cuda/math.cuh"
inline float min(float a, float b) { return a < b ? a : b; }
#include "include/cuda/brdf.cuh"
#define KOBRA_OPTIX_LIGHTING_H_IMPL
#include "include/optix/lighting.cuh"

using namespace kobra::cuda;
using namespace kobra::optix;

static uint64_t lcg_state = 0x243F6A8885A308D3ull;
static float frand(float lo, float hi)
{
	lcg_state = lcg_state * 6364136223846793005ull + 1442695040888963407ull;
	uint32_t bits = (uint32_t)(lcg_state >> 40); /* 24 bits */
	float u = (float)bits / 16777216.0f;
	return lo + (hi - lo) * u;
}

static void pf(float v, bool comma = true) { printf("%.9g%s", v, comma ? ", " : ""); }
static void p3(float3 v, bool comma = true) { printf("[%.9g, %.9g, %.9g]%s", v.x, v.y, v.z, comma ? ", " : ""); }

int main()
{
	printf("{\n");
	/* RNG streams */
	printf("\"rng\": [\n");
	float seeds[][3] = {{1, 2, 3}, {0, 0, 0}, {0.5f, 0.25f, 0.125f}, {123.0f, -7.5f, 1e-3f}};
	for (int s = 0; s < 4; s++) {
		float3 seed = make_float3(seeds[s][0], seeds[s][1], seeds[s][2]);
		printf(" {\"seed\": "); p3(seed, false); printf(", \"draws\": [");
		for (int i = 0; i < 16; i++) {
			float u = rand_uniform(seed);
			printf("[%.9g, %.9g, %.9g, %.9g]%s", u, seed.x, seed.y, seed.z, i < 15 ? ", " : "");
		}
		printf("]}%s\n", s < 3 ? "," : "");
	}
	/* stream from integer bit-pattern seeds {p ^ f, p, f} */
	printf("],\n\"rng_bits\": [\n");
	unsigned int pix[][2] = {{0, 0}, {1, 0}, {65535, 3}, {2073599, 17}};
	for (int s = 0; s < 4; s++) {
		uint3 b = make_uint3(pix[s][0] ^ pix[s][1], pix[s][0], pix[s][1]);
		float3 seed = *reinterpret_cast<float3 *>(&b);
		printf(" {\"pixel\": %u, \"stream\": %u, \"draws\": [", pix[s][0], pix[s][1]);
		for (int i = 0; i < 8; i++) {
			float3 r = rand_uniform_3f(seed);
			printf("[%.9g, %.9g, %.9g]%s", r.x, r.y, r.z, i < 7 ? ", " : "");
		}
		printf("]}%s\n", s < 3 ? "," : "");
	}
	/* triangle tests */
	printf("],\n\"intersect\": [\n");
	for (int i = 0; i < 400; i++) {
		float3 v1 = make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1));
		float3 v2 = make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1));
		float3 v3 = make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1));
		float3 o = make_float3(frand(-3, 3), frand(-3, 3), frand(-3, 3));
		float3 target = (v1 + v2 + v3) / 3.0f + make_float3(frand(-0.3f, 0.3f), frand(-0.3f, 0.3f), frand(-0.3f, 0.3f));
		float3 d = normalize(target - o);
		float t = intersects_triangle(v1, v2, v3, o, d);
		printf(" {\"v\": ["); p3(v1); p3(v2); p3(v3, false);
		printf("], \"o\": "); p3(o); printf("\"d\": "); p3(d, false);
		printf(", \"t\": %.9g}%s\n", t, i < 399 ? "," : "");
	}
	/* area lights */
	printf("],\n\"lights\": [\n");
	for (int i = 0; i < 64; i++) {
		TriangleLight l;
		l.a = make_float3(frand(-2, 2), frand(-2, 2), frand(-2, 2));
		l.ab = make_float3(frand(-0.5f, 0.5f), frand(-0.5f, 0.5f), frand(-0.5f, 0.5f));
		l.ac = make_float3(frand(-0.5f, 0.5f), frand(-0.5f, 0.5f), frand(-0.5f, 0.5f));
		l.intensity = make_float3(1, 2, 3);
		float3 seed = make_float3(frand(0, 1), frand(0, 1), frand(0, 1));
		float3 seed0 = seed;
		float3 p = sample_area_light(l, seed);
		printf(" {\"a\": "); p3(l.a); printf("\"ab\": "); p3(l.ab); printf("\"ac\": "); p3(l.ac);
		printf("\"seed\": "); p3(seed0); printf("\"point\": "); p3(p); printf("\"area\": %.9g, \"normal\": ", l.area());
		p3(l.normal(), false); printf("}%s\n", i < 63 ? "," : "");
	}
	/* BRDF evaluation and sampling */
	printf("],\n\"brdf\": [\n");
	for (int i = 0; i < 200; i++) {
		SurfaceHit sh;
		float kd = frand(0.1f, 0.9f);
		bool ggx = i % 2 == 1;
		sh.mat.diffuse = make_float3(kd, kd * 0.8f, kd * 0.6f);
		float ks = ggx ? frand(0.2f, 0.9f) : 0.0f;
		sh.mat.specular = make_float3(ks, ks, ks);
		sh.mat.emission = make_float3(0, 0, 0);
		sh.mat.ambient = make_float3(0, 0, 0);
		sh.mat.shininess = 0;
		sh.mat.roughness = ggx ? frand(0.05f, 0.8f) : 1.0f;
		sh.mat.refraction = 1;
		sh.mat.type = eDiffuse;
		sh.entering = true;
		sh.n = normalize(make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1)));
		sh.wo = normalize(sh.n + make_float3(frand(-0.9f, 0.9f), frand(-0.9f, 0.9f), frand(-0.9f, 0.9f)));
		sh.x = make_float3(0, 0, 0);
		float3 wi_fixed = normalize(sh.n + make_float3(frand(-0.9f, 0.9f), frand(-0.9f, 0.9f), frand(-0.9f, 0.9f)));
		float3 f_fixed = brdf(sh, wi_fixed, eDiffuse);
		float pdf_fixed = pdf(sh, wi_fixed, eDiffuse);
		float3 seed = make_float3(frand(0, 1), frand(0, 1), frand(0, 1));
		float3 seed0 = seed;
		float3 wi;
		float in_pdf = 0;
		Shading out;
		float3 f = eval(sh, wi, in_pdf, out, seed);
		printf(" {\"diffuse\": "); p3(sh.mat.diffuse); printf("\"specular\": "); p3(sh.mat.specular);
		printf("\"roughness\": %.9g, \"n\": ", sh.mat.roughness); p3(sh.n); printf("\"wo\": "); p3(sh.wo);
		printf("\"wi_fixed\": "); p3(wi_fixed); printf("\"f_fixed\": "); p3(f_fixed);
		printf("\"pdf_fixed\": %.9g, \"seed\": ", pdf_fixed); p3(seed0);
		printf("\"f\": "); p3(f); printf("\"wi\": "); p3(wi); printf("\"pdf\": %.9g, \"seed_after\": ", in_pdf);
		p3(seed, false); printf("}%s\n", i < 199 ? "," : "");
	}
	/* rotate */
	printf("],\n\"rotate\": [\n");
	for (int i = 0; i < 64; i++) {
		float3 s = make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1));
		float3 n = normalize(make_float3(frand(-1, 1), frand(-1, 1), frand(-1, 1)));
		if (i == 0) n = make_float3(0, 1, 0);
		float3 r = rotate(s, n);
		printf(" {\"s\": "); p3(s); printf("\"n\": "); p3(n); printf("\"r\": "); p3(r, false);
		printf("}%s\n", i < 63 ? "," : "");
	}
	printf("]\n}\n");
	return 0;
}
