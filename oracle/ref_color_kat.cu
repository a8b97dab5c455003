/*
 * ref_color_kat.cu -- known answers of the reference's HDR -> LDR mapping.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) with nvcc,
 * host code only, against the reference checkout (REFERENCE=<path>), into
 * oracle/_ref/ref_color_kat.  It includes include/cuda/color.cuh unmodified
 * and prints, for a sweep of HDR colours, the packed 32-bit pixel that
 * make_color + to_ui32 give for each tonemapping (0 ACES, 1 sRGB).  nvcc is
 * needed because color.cuh also holds the hdr_to_ldr kernel launch.  One
 * shim: color.cuh includes cast.cuh, which includes glm (not vendored in the
 * checkout) for glm::vec3 only; oracle/shim/glm/glm.hpp declares that type.
 * tests/golden/gen_golden.py merges the JSON into reference_kat.json.
 */
#include <cstdio>
#include <cstdint>

#include "include/cuda/color.cuh"

using namespace kobra::cuda;

static uint64_t state = 0x13198A2E03707344ull;
static float frand(float lo, float hi)
{
	state = state * 6364136223846793005ull + 1442695040888963407ull;
	uint32_t bits = (uint32_t)(state >> 40);
	return lo + (hi - lo) * ((float)bits / 16777216.0f);
}

int main()
{
	const float fixed[] = {0.0f, 1e-6f, 0.001f, 0.0031307f, 0.0031308f, 0.0031309f, 0.01f, 0.1f, 0.18f, 0.5f,
		0.99f, 1.0f, 1.5f, 4.0f, 16.0f, 100.0f, 1e4f};
	const int nf = sizeof(fixed) / sizeof(fixed[0]);
	printf("{\"tonemap\": [\n");
	const int total = nf + 400;
	for (int i = 0; i < total; i++) {
		float3 c;
		if (i < nf)
			c = make_float3(fixed[i], fixed[i] * 0.5f, fixed[i] * 2.0f);
		else {
			float s = frand(-3.0f, 2.0f); /* log10 of the scale: 1e-3 .. 100 */
			float k = powf(10.0f, s);
			c = make_float3(k * frand(0.0f, 1.0f), k * frand(0.0f, 1.0f), k * frand(0.0f, 1.0f));
		}
		uint32_t aces = to_ui32(make_color(c, 0));
		uint32_t srgb = to_ui32(make_color(c, 1));
		printf(" {\"c\": [%.9g, %.9g, %.9g], \"aces\": %u, \"srgb\": %u}%s\n", c.x, c.y, c.z, aces, srgb,
			i < total - 1 ? "," : "");
	}
	printf("]}\n");
	return 0;
}
