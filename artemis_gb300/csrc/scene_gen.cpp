/*
 * scene_gen.cpp -- seeded procedural scenes (the reference's benchmark
 * scenes are not available; these stand in with the shapes, sizes and value
 * distributions of the benchmark configurations).
 *
 * Only integer hashing and IEEE + - * / sqrt are used, so a (name, seed)
 * pair gives the same bits on x86-64 and aarch64.
 */
#include <math.h>
#include <string.h>

#include <map>
#include <string>
#include <utility>

#include "kgr_internal.h"

namespace kgr {
namespace {

struct Rng {
	uint64_t s;
	explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull) {}
	uint64_t next()
	{
		/* splitmix64 */
		uint64_t z = (s += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		return z ^ (z >> 31);
	}
	/* uniform in [0, 1) with 24 random bits */
	float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
	float uniform(float lo, float hi) { return lo + (hi - lo) * uniform(); }
};

struct V3 {
	float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 normalize(V3 a) { float inv = 1.0f / sqrtf(dot(a, a)); return a * inv; }

/* three draws in x, y, z order: the order in which a function's arguments
 * are evaluated is unspecified in C++ (GCC takes them right to left on
 * x86-64), so multi-draw values are sequenced through here */
V3 draw3(Rng &r, float lo, float hi)
{
	float x = r.uniform(lo, hi);
	float y = r.uniform(lo, hi);
	float z = r.uniform(lo, hi);
	return v3(x, y, z);
}

/* uniform direction by rejection from the cube (no transcendentals) */
V3 random_unit(Rng &r)
{
	for (;;) {
		V3 v = draw3(r, -1, 1);
		float l2 = dot(v, v);
		if (l2 > 1e-4f && l2 <= 1.0f)
			return normalize(v);
	}
}

/* exp(x) by halving and squaring of a Taylor series (generator use only) */
float gen_exp(float x)
{
	int k = 0;
	float y = x;
	while (y > 0.125f || y < -0.125f) {
		y *= 0.5f;
		k++;
	}
	float e = 1.0f + y * (1.0f + y * (0.5f + y * (1.0f / 6 + y * (1.0f / 24 + y * (1.0f / 120)))));
	while (k-- > 0)
		e = e * e;
	return e;
}

struct Builder {
	kgr_generated *g;
	uint32_t add_vertex(V3 p, V3 n)
	{
		g->positions.insert(g->positions.end(), {p.x, p.y, p.z});
		g->normals.insert(g->normals.end(), {n.x, n.y, n.z});
		return (uint32_t)(g->positions.size() / 3 - 1);
	}
	void add_tri(uint32_t a, uint32_t b, uint32_t c, uint32_t mat)
	{
		g->indices.insert(g->indices.end(), {a, b, c});
		g->material_indices.push_back(mat);
	}
	/* flat triangle with its own three vertices */
	void flat_tri(V3 a, V3 b, V3 c, uint32_t mat)
	{
		V3 n = normalize(cross(b - a, c - a));
		uint32_t i = add_vertex(a, n), j = add_vertex(b, n), k = add_vertex(c, n);
		add_tri(i, j, k, mat);
	}
	void quad(V3 a, V3 b, V3 c, V3 d, uint32_t mat)
	{
		flat_tri(a, b, c, mat);
		flat_tri(a, c, d, mat);
	}
	uint32_t material(V3 diffuse, V3 specular, V3 emission, float roughness, int type)
	{
		kgr_material m;
		memset(&m, 0, sizeof(m));
		m.diffuse[0] = diffuse.x; m.diffuse[1] = diffuse.y; m.diffuse[2] = diffuse.z;
		m.specular[0] = specular.x; m.specular[1] = specular.y; m.specular[2] = specular.z;
		m.emission[0] = emission.x; m.emission[1] = emission.y; m.emission[2] = emission.z;
		m.roughness = roughness;
		m.refraction = 1.0f;
		m.type = type;
		g->materials.push_back(m);
		return (uint32_t)g->materials.size() - 1;
	}
	uint32_t lambert(Rng &r)
	{
		V3 kd = draw3(r, 0.1f, 0.9f);
		return material(kd, v3(0, 0, 0), v3(0, 0, 0), 1.0f, KGR_SHADING_DIFFUSE);
	}
	uint32_t ggx(Rng &r)
	{
		V3 kd = draw3(r, 0.05f, 0.5f);
		float ks = r.uniform(0.2f, 0.9f);
		float rough = r.uniform(0.05f, 0.8f);
		return material(kd, v3(ks, ks, ks), v3(0, 0, 0), rough, KGR_SHADING_DIFFUSE);
	}
	uint32_t emitter(float radiance)
	{
		return material(v3(0, 0, 0), v3(0, 0, 0), v3(radiance, radiance, radiance), 1.0f,
			KGR_SHADING_EMISSIVE);
	}
};

/* box [-2,2]^3 (12 tris) + 4096 random triangles with centroids in
 * [-1.5,1.5]^3 and edges in [0.05,0.2] + 64 emissive ceiling quads with
 * radiance in [1,10]; Lambertian albedo in [0.1,0.9]. */
void gen_box4k(kgr_generated *g, uint64_t seed, int random_tris)
{
	Rng r(seed);
	Builder b{g};
	const float S = 2.0f;
	V3 p[8];
	for (int i = 0; i < 8; i++)
		p[i] = v3(i & 1 ? S : -S, i & 2 ? S : -S, i & 4 ? S : -S);
	int faces[6][4] = {{0, 1, 3, 2}, {4, 6, 7, 5}, {0, 4, 5, 1}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 5, 7, 3}};
	for (int f = 0; f < 6; f++) {
		uint32_t m = b.lambert(r);
		b.quad(p[faces[f][0]], p[faces[f][1]], p[faces[f][2]], p[faces[f][3]], m);
	}
	for (int i = 0; i < random_tris; i++) {
		V3 c = draw3(r, -1.5f, 1.5f);
		V3 u = random_unit(r);
		V3 w = random_unit(r);
		V3 q = w - u * dot(w, u);
		if (dot(q, q) < 1e-6f)
			q = cross(u, fabsf(u.x) < 0.9f ? v3(1, 0, 0) : v3(0, 1, 0));
		q = normalize(q);
		float l1 = r.uniform(0.05f, 0.2f), l2 = r.uniform(0.05f, 0.2f);
		float ct = r.uniform(-0.5f, 0.5f);
		float st = sqrtf(1.0f - ct * ct);
		V3 a = v3(0, 0, 0), bb = u * l1, cc = (u * ct + q * st) * l2;
		V3 cen = (a + bb + cc) * (1.0f / 3.0f);
		b.flat_tri(a - cen + c, bb - cen + c, cc - cen + c, b.lambert(r));
	}
	/* 8 x 8 emissive quads 0.2 x 0.2 just below the ceiling, facing down */
	for (int i = 0; i < 8; i++)
		for (int j = 0; j < 8; j++) {
			float x0 = -1.6f + 0.4f * i + 0.1f, z0 = -1.6f + 0.4f * j + 0.1f;
			float y = 1.99f;
			uint32_t m = b.emitter(r.uniform(1.0f, 10.0f));
			b.quad(v3(x0, y, z0), v3(x0 + 0.2f, y, z0), v3(x0 + 0.2f, y, z0 + 0.2f), v3(x0, y, z0 + 0.2f), m);
		}
	g->eye[0] = 0; g->eye[1] = 0; g->eye[2] = 1.9f;
	g->target[0] = 0; g->target[1] = 0; g->target[2] = 0.9f;
	g->fov = 60.0f;
}

/* value noise on a G x G lattice with smoothstep interpolation */
struct Noise {
	int G;
	std::vector<float> v;
	Noise(int g, Rng &r) : G(g), v((size_t)(g + 1) * (g + 1))
	{
		for (float &x : v)
			x = r.uniform(-1.0f, 1.0f);
	}
	float at(float u, float w) const /* u, w in [0, 1] */
	{
		float fu = u * G, fw = w * G;
		int i = (int)fu, j = (int)fw;
		i = i < 0 ? 0 : (i >= G ? G - 1 : i);
		j = j < 0 ? 0 : (j >= G ? G - 1 : j);
		float tu = fu - (float)i, tw = fw - (float)j;
		tu = tu * tu * (3.0f - 2.0f * tu);
		tw = tw * tw * (3.0f - 2.0f * tw);
		float a = v[(size_t)j * (G + 1) + i], b = v[(size_t)j * (G + 1) + i + 1];
		float c = v[(size_t)(j + 1) * (G + 1) + i], d = v[(size_t)(j + 1) * (G + 1) + i + 1];
		float ab = a + (b - a) * tu, cd = c + (d - c) * tu;
		return ab + (cd - ab) * tw;
	}
};

/* unit icosphere subdivided twice: 162 vertices, 320 triangles */
void icosphere(std::vector<V3> &verts, std::vector<uint32_t> &tris)
{
	const float t = 1.61803398875f;
	V3 base[12] = {v3(-1, t, 0), v3(1, t, 0), v3(-1, -t, 0), v3(1, -t, 0), v3(0, -1, t), v3(0, 1, t),
		v3(0, -1, -t), v3(0, 1, -t), v3(t, 0, -1), v3(t, 0, 1), v3(-t, 0, -1), v3(-t, 0, 1)};
	uint32_t f[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
		{11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9},
		{4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
	verts.clear();
	for (V3 v : base)
		verts.push_back(normalize(v));
	tris.assign(&f[0][0], &f[0][0] + 60);
	for (int level = 0; level < 2; level++) {
		std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
		auto midpoint = [&](uint32_t a, uint32_t b) {
			auto key = std::make_pair(a < b ? a : b, a < b ? b : a);
			auto it = mid.find(key);
			if (it != mid.end())
				return it->second;
			V3 m = normalize((verts[a] + verts[b]) * 0.5f);
			verts.push_back(m);
			uint32_t id = (uint32_t)verts.size() - 1;
			mid[key] = id;
			return id;
		};
		std::vector<uint32_t> nt;
		for (size_t i = 0; i < tris.size(); i += 3) {
			uint32_t a = tris[i], b = tris[i + 1], c = tris[i + 2];
			uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
			uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
			nt.insert(nt.end(), add, add + 12);
		}
		tris.swap(nt);
	}
}

/* height field of grid x grid quads over [-2,2]^2 with value-noise
 * amplitude 0.3, `spheres` icospheres (radius in [0.02,0.1]) resting on it,
 * and light_quads emissive quads at y = 1.2 facing down.  Materials: a
 * palette of 32 Lambertian and 32 GGX (roughness in [0.05,0.8]) entries. */
void gen_terrain(kgr_generated *g, uint64_t seed, int grid, int spheres, int light_quads, bool log_radiance)
{
	Rng r(seed);
	Builder b{g};
	std::vector<uint32_t> palette;
	for (int i = 0; i < 64; i++)
		palette.push_back(i % 2 ? b.ggx(r) : b.lambert(r));
	Noise n1(16, r), n2(64, r);
	const float H = 0.3f;
	auto height = [&](float u, float w) { return H * (n1.at(u, w) + 0.5f * n2.at(u, w)) * (1.0f / 1.5f) - 0.5f; };
	int N = grid;
	float step = 4.0f / (float)N;
	std::vector<float> hgt((size_t)(N + 1) * (N + 1));
	for (int j = 0; j <= N; j++)
		for (int i = 0; i <= N; i++)
			hgt[(size_t)j * (N + 1) + i] = height((float)i / N, (float)j / N);
	uint32_t base = (uint32_t)(g->positions.size() / 3);
	for (int j = 0; j <= N; j++)
		for (int i = 0; i <= N; i++) {
			int i0 = i > 0 ? i - 1 : i, i1 = i < N ? i + 1 : i;
			int j0 = j > 0 ? j - 1 : j, j1 = j < N ? j + 1 : j;
			float dx = (hgt[(size_t)j * (N + 1) + i1] - hgt[(size_t)j * (N + 1) + i0]) / ((float)(i1 - i0) * step);
			float dz = (hgt[(size_t)j1 * (N + 1) + i] - hgt[(size_t)j0 * (N + 1) + i]) / ((float)(j1 - j0) * step);
			V3 p = v3(-2.0f + step * i, hgt[(size_t)j * (N + 1) + i], -2.0f + step * j);
			b.add_vertex(p, normalize(v3(-dx, 1.0f, -dz)));
		}
	int patches = 8;
	for (int j = 0; j < N; j++)
		for (int i = 0; i < N; i++) {
			int pi = i * patches / N, pj = j * patches / N;
			uint32_t m = palette[(uint32_t)(pj * patches + pi) * 7 % 64];
			uint32_t v00 = base + (uint32_t)(j * (N + 1) + i), v10 = v00 + 1;
			uint32_t v01 = v00 + (uint32_t)(N + 1), v11 = v01 + 1;
			b.add_tri(v00, v01, v11, m);
			b.add_tri(v00, v11, v10, m);
		}
	std::vector<V3> sv;
	std::vector<uint32_t> st;
	icosphere(sv, st);
	for (int s = 0; s < spheres; s++) {
		float x = r.uniform(-1.9f, 1.9f), z = r.uniform(-1.9f, 1.9f);
		float rad = r.uniform(0.02f, 0.1f);
		float y = height((x + 2.0f) * 0.25f, (z + 2.0f) * 0.25f) + rad * r.uniform(0.2f, 1.0f);
		uint32_t m = palette[(uint32_t)(r.next() % 64)];
		uint32_t vb = (uint32_t)(g->positions.size() / 3);
		V3 c = v3(x, y, z);
		for (V3 u : sv)
			b.add_vertex(c + u * rad, u);
		for (size_t k = 0; k < st.size(); k += 3)
			b.add_tri(vb + st[k], vb + st[k + 1], vb + st[k + 2], m);
	}
	/* emissive quads on a grid at y = 1.2, facing down */
	int cols = 1;
	while (cols * cols < light_quads)
		cols++;
	int rows = (light_quads + cols - 1) / cols;
	float cell_x = 3.6f / cols, cell_z = 3.6f / rows;
	float size = (cell_x < cell_z ? cell_x : cell_z) * 0.4f;
	for (int k = 0; k < light_quads; k++) {
		int i = k % cols, j = k / cols;
		float x0 = -1.8f + cell_x * i + (cell_x - size) * 0.5f;
		float z0 = -1.8f + cell_z * j + (cell_z - size) * 0.5f;
		float y = 1.2f;
		float rad = log_radiance ? 0.1f * gen_exp(r.uniform(0.0f, 6.90775528f)) : r.uniform(1.0f, 10.0f);
		uint32_t m = b.emitter(rad);
		b.quad(v3(x0, y, z0), v3(x0 + size, y, z0), v3(x0 + size, y, z0 + size), v3(x0, y, z0 + size), m);
	}
	g->eye[0] = 0; g->eye[1] = 1.0f; g->eye[2] = 2.4f;
	g->target[0] = 0; g->target[1] = -0.3f; g->target[2] = 0;
	g->fov = 60.0f;
}

/* a few triangles for unit tests: a floor, a blocker, a light */
void gen_tiny(kgr_generated *g, uint64_t seed)
{
	Rng r(seed);
	Builder b{g};
	uint32_t m = b.lambert(r);
	b.quad(v3(-1, 0, -1), v3(1, 0, -1), v3(1, 0, 1), v3(-1, 0, 1), m);
	b.flat_tri(v3(-0.3f, 0.5f, -0.3f), v3(0.3f, 0.5f, -0.3f), v3(0, 0.5f, 0.3f), b.ggx(r));
	uint32_t e = b.emitter(5.0f);
	b.quad(v3(-0.2f, 1.5f, -0.2f), v3(0.2f, 1.5f, -0.2f), v3(0.2f, 1.5f, 0.2f), v3(-0.2f, 1.5f, 0.2f), e);
	g->eye[0] = 0; g->eye[1] = 1.0f; g->eye[2] = 2.5f;
	g->target[0] = 0; g->target[1] = 0.2f; g->target[2] = 0;
	g->fov = 60.0f;
}

} /* namespace */

void generate_scene(const std::string &name, uint64_t seed, kgr_generated *g)
{
	if (name == "box4k")
		gen_box4k(g, seed, 4096);
	else if (name == "box64")
		gen_box4k(g, seed, 64);
	else if (name == "terrain")
		gen_terrain(g, seed, 512, 2000, 512, false);
	else if (name == "terrain_s")
		gen_terrain(g, seed, 256, 400, 512, false);
	else if (name == "terrain_m")
		gen_terrain(g, seed, 512, 1500, 512, false);
	else if (name == "terrain_l")
		gen_terrain(g, seed, 1024, 6000, 32768, true);
	else if (name == "tiny")
		gen_tiny(g, seed);
	else
		throw Error(KGR_ERR_INVALID_ARGUMENT, "unknown procedural scene: " + name);
}

} /* namespace kgr */
