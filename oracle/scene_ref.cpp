/*
 * scene_ref.cpp -- the oracle's own scene inputs (TEST INFRASTRUCTURE).
 *
 * The CPU reference arm of the benchmark must not load the product library,
 * so everything it needs besides the per-pixel path lives here, written
 * independently of the product's sources and checked against them by the
 * CPU tests (tests/test_oracle_scene.py):
 *
 *  - the seeded procedural scenes that stand in for the reference's
 *    benchmark scenes (the box scene: a [-2,2]^3 box, random triangles and
 *    64 emissive ceiling quads; the terrain: a value-noise height field,
 *    icospheres and emissive quads).  Only integer hashing and IEEE
 *    + - * / sqrt are used, so a (name, seed) pair gives the same bits on
 *    x86-64 and aarch64;
 *  - a binned-SAH builder with leaves of at most max_leaf triangles (32
 *    centroid bins per axis, stable partition), serialised in the threaded
 *    layout of serialize() (source/bvh.cpp:213-260) with a leaf of k
 *    triangles written as k one-triangle leaf records chained by their miss
 *    links;
 *  - the triangle lights ArmadaRTX derives from emissive submeshes
 *    (source/amadeus/armada.cu:98-212): {a, b - a, c - a, emission} in
 *    triangle order;
 *  - the pinhole camera frame of uvw_frame (include/camera.hpp:45-63).
 */
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "oracle.h"

namespace {

/* ------------------------------------------------------------ generator -- */

struct Stream {
	uint64_t state;
	explicit Stream(uint64_t seed) : state(seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull) {}
	uint64_t bits()
	{
		/* splitmix64 (Steele, Lea, Flood 2014) */
		state += 0x9E3779B97F4A7C15ull;
		uint64_t z = state;
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		return z ^ (z >> 31);
	}
	float unit() { return (float)(bits() >> 40) * (1.0f / 16777216.0f); } /* 24 bits in [0, 1) */
	float range(float lo, float hi) { return lo + (hi - lo) * unit(); }
};

struct P3 {
	float x, y, z;
};
P3 p3(float x, float y, float z) { return P3{x, y, z}; }
P3 add(P3 a, P3 b) { return p3(a.x + b.x, a.y + b.y, a.z + b.z); }
P3 sub(P3 a, P3 b) { return p3(a.x - b.x, a.y - b.y, a.z - b.z); }
P3 scale(P3 a, float s) { return p3(a.x * s, a.y * s, a.z * s); }
float dotp(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
P3 crossp(P3 a, P3 b) { return p3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
P3 unitv(P3 a)
{
	float r = 1.0f / sqrtf(dotp(a, a));
	return scale(a, r);
}

/* direction uniform on the sphere, by rejection from the cube */
P3 sphere_dir(Stream &s)
{
	while (true) {
		float x = s.range(-1, 1), y = s.range(-1, 1), z = s.range(-1, 1);
		P3 v = p3(x, y, z);
		float l2 = dotp(v, v);
		if (l2 > 1e-4f && l2 <= 1.0f)
			return unitv(v);
	}
}

/* e^x for the log-uniform light radiance: x is halved until |x| <= 1/8, a
 * degree-5 Taylor polynomial is evaluated there and squared back up */
float exp_halving(float x)
{
	int halvings = 0;
	while (x > 0.125f || x < -0.125f) {
		x *= 0.5f;
		halvings++;
	}
	float e = 1.0f + x * (1.0f + x * (0.5f + x * (1.0f / 6 + x * (1.0f / 24 + x * (1.0f / 120)))));
	for (; halvings > 0; halvings--)
		e = e * e;
	return e;
}

struct Mesh {
	std::vector<float> pos, nrm;
	std::vector<uint32_t> idx, mat;
	std::vector<kgr_material> mats;
	float eye[3], target[3], fov;

	uint32_t vertex(P3 p, P3 n)
	{
		float v[3] = {p.x, p.y, p.z}, m[3] = {n.x, n.y, n.z};
		pos.insert(pos.end(), v, v + 3);
		nrm.insert(nrm.end(), m, m + 3);
		return (uint32_t)(pos.size() / 3) - 1;
	}
	void tri(uint32_t a, uint32_t b, uint32_t c, uint32_t m)
	{
		uint32_t t[3] = {a, b, c};
		idx.insert(idx.end(), t, t + 3);
		mat.push_back(m);
	}
	void facet(P3 a, P3 b, P3 c, uint32_t m)
	{
		P3 n = unitv(crossp(sub(b, a), sub(c, a)));
		uint32_t i = vertex(a, n);
		uint32_t j = vertex(b, n);
		uint32_t k = vertex(c, n);
		tri(i, j, k, m);
	}
	uint32_t material(float kd[3], float ks[3], float ke[3], float roughness, int32_t type)
	{
		kgr_material m;
		memset(&m, 0, sizeof(m));
		memcpy(m.diffuse, kd, 12);
		memcpy(m.specular, ks, 12);
		memcpy(m.emission, ke, 12);
		m.roughness = roughness;
		m.refraction = 1.0f;
		m.type = type;
		mats.push_back(m);
		return (uint32_t)mats.size() - 1;
	}
	uint32_t diffuse(Stream &s)
	{
		float kd[3];
		kd[0] = s.range(0.1f, 0.9f);
		kd[1] = s.range(0.1f, 0.9f);
		kd[2] = s.range(0.1f, 0.9f);
		float zero[3] = {0, 0, 0};
		return material(kd, zero, zero, 1.0f, KGR_SHADING_DIFFUSE);
	}
	uint32_t glossy(Stream &s)
	{
		float kd[3];
		kd[0] = s.range(0.05f, 0.5f);
		kd[1] = s.range(0.05f, 0.5f);
		kd[2] = s.range(0.05f, 0.5f);
		float k = s.range(0.2f, 0.9f);
		float roughness = s.range(0.05f, 0.8f);
		float ks[3] = {k, k, k}, zero[3] = {0, 0, 0};
		return material(kd, ks, zero, roughness, KGR_SHADING_DIFFUSE);
	}
	uint32_t light(float radiance)
	{
		float zero[3] = {0, 0, 0}, ke[3] = {radiance, radiance, radiance};
		return material(zero, zero, ke, 1.0f, KGR_SHADING_EMISSIVE);
	}
	void camera(float ex, float ey, float ez, float tx, float ty, float tz)
	{
		eye[0] = ex; eye[1] = ey; eye[2] = ez;
		target[0] = tx; target[1] = ty; target[2] = tz;
		fov = 60.0f;
	}
};

void box_scene(Mesh &m, uint64_t seed, int clutter)
{
	Stream s(seed);
	P3 corner[8];
	for (int i = 0; i < 8; i++)
		corner[i] = p3((i & 1) ? 2.0f : -2.0f, (i & 2) ? 2.0f : -2.0f, (i & 4) ? 2.0f : -2.0f);
	static const int face[6][4] = {{0, 1, 3, 2}, {4, 6, 7, 5}, {0, 4, 5, 1}, {2, 3, 7, 6}, {0, 2, 6, 4}, {1, 5, 7, 3}};
	for (const auto &f : face) {
		uint32_t mt = m.diffuse(s);
		m.facet(corner[f[0]], corner[f[1]], corner[f[2]], mt);
		m.facet(corner[f[0]], corner[f[2]], corner[f[3]], mt);
	}
	for (int i = 0; i < clutter; i++) {
		float cx = s.range(-1.5f, 1.5f);
		float cy = s.range(-1.5f, 1.5f);
		float cz = s.range(-1.5f, 1.5f);
		P3 c = p3(cx, cy, cz);
		P3 u = sphere_dir(s);
		P3 w = sphere_dir(s);
		P3 q = sub(w, scale(u, dotp(w, u)));
		if (dotp(q, q) < 1e-6f)
			q = crossp(u, fabsf(u.x) < 0.9f ? p3(1, 0, 0) : p3(0, 1, 0));
		q = unitv(q);
		float l1 = s.range(0.05f, 0.2f);
		float l2 = s.range(0.05f, 0.2f);
		float ct = s.range(-0.5f, 0.5f);
		float st = sqrtf(1.0f - ct * ct);
		P3 a = p3(0, 0, 0), b = scale(u, l1), d = scale(add(scale(u, ct), scale(q, st)), l2);
		P3 mid = scale(add(add(a, b), d), 1.0f / 3.0f);
		uint32_t mt = m.diffuse(s);
		m.facet(add(sub(a, mid), c), add(sub(b, mid), c), add(sub(d, mid), c), mt);
	}
	/* an 8 x 8 grid of 0.2 x 0.2 emitters just below the ceiling, facing down */
	for (int i = 0; i < 8; i++)
		for (int j = 0; j < 8; j++) {
			float x0 = -1.6f + 0.4f * i + 0.1f, z0 = -1.6f + 0.4f * j + 0.1f, y = 1.99f;
			uint32_t mt = m.light(s.range(1.0f, 10.0f));
			P3 a = p3(x0, y, z0), b = p3(x0 + 0.2f, y, z0), c = p3(x0 + 0.2f, y, z0 + 0.2f), d = p3(x0, y, z0 + 0.2f);
			m.facet(a, b, c, mt);
			m.facet(a, c, d, mt);
		}
	m.camera(0, 0, 1.9f, 0, 0, 0.9f);
}

/* value noise on a lattice of n x n cells with smoothstep weights */
struct Lattice {
	int n;
	std::vector<float> val;
	Lattice(int cells, Stream &s) : n(cells), val((size_t)(cells + 1) * (cells + 1))
	{
		for (size_t i = 0; i < val.size(); i++)
			val[i] = s.range(-1.0f, 1.0f);
	}
	float operator()(float u, float w) const
	{
		float fu = u * n, fw = w * n;
		int i = std::min(std::max((int)fu, 0), n - 1);
		int j = std::min(std::max((int)fw, 0), n - 1);
		float su = fu - (float)i, sw = fw - (float)j;
		su = su * su * (3.0f - 2.0f * su);
		sw = sw * sw * (3.0f - 2.0f * sw);
		const float *row0 = &val[(size_t)j * (n + 1)], *row1 = &val[(size_t)(j + 1) * (n + 1)];
		float lo = row0[i] + (row0[i + 1] - row0[i]) * su;
		float hi = row1[i] + (row1[i + 1] - row1[i]) * su;
		return lo + (hi - lo) * sw;
	}
};

/* twice-subdivided icosahedron on the unit sphere: 162 vertices, 320 faces */
void unit_icosphere(std::vector<P3> &v, std::vector<uint32_t> &f)
{
	const float g = 1.61803398875f;
	const P3 seed_v[12] = {p3(-1, g, 0), p3(1, g, 0), p3(-1, -g, 0), p3(1, -g, 0), p3(0, -1, g), p3(0, 1, g),
		p3(0, -1, -g), p3(0, 1, -g), p3(g, 0, -1), p3(g, 0, 1), p3(-g, 0, -1), p3(-g, 0, 1)};
	static const uint32_t seed_f[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
		11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10,
		8, 6, 7, 9, 8, 1};
	v.clear();
	for (const P3 &p : seed_v)
		v.push_back(unitv(p));
	f.assign(seed_f, seed_f + 60);
	for (int pass = 0; pass < 2; pass++) {
		std::map<std::pair<uint32_t, uint32_t>, uint32_t> split;
		auto middle = [&](uint32_t a, uint32_t b) -> uint32_t {
			std::pair<uint32_t, uint32_t> key(std::min(a, b), std::max(a, b));
			auto found = split.find(key);
			if (found != split.end())
				return found->second;
			v.push_back(unitv(scale(add(v[a], v[b]), 0.5f)));
			uint32_t id = (uint32_t)v.size() - 1;
			split.emplace(key, id);
			return id;
		};
		std::vector<uint32_t> out;
		out.reserve(f.size() * 4);
		for (size_t t = 0; t < f.size(); t += 3) {
			uint32_t a = f[t], b = f[t + 1], c = f[t + 2];
			uint32_t ab = middle(a, b);
			uint32_t bc = middle(b, c);
			uint32_t ca = middle(c, a);
			const uint32_t four[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
			out.insert(out.end(), four, four + 12);
		}
		f.swap(out);
	}
}

void terrain_scene(Mesh &m, uint64_t seed, int cells, int spheres, int emitters, bool log_radiance)
{
	Stream s(seed);
	std::vector<uint32_t> palette;
	for (int i = 0; i < 64; i++)
		palette.push_back(i % 2 ? m.glossy(s) : m.diffuse(s));
	Lattice coarse(16, s), fine(64, s);
	auto height = [&](float u, float w) {
		return 0.3f * (coarse(u, w) + 0.5f * fine(u, w)) * (1.0f / 1.5f) - 0.5f;
	};
	const int N = cells;
	const float step = 4.0f / (float)N;
	std::vector<float> h((size_t)(N + 1) * (N + 1));
	for (int j = 0; j <= N; j++)
		for (int i = 0; i <= N; i++)
			h[(size_t)j * (N + 1) + i] = height((float)i / N, (float)j / N);
	auto H = [&](int i, int j) { return h[(size_t)j * (N + 1) + i]; };
	uint32_t first = (uint32_t)(m.pos.size() / 3);
	for (int j = 0; j <= N; j++)
		for (int i = 0; i <= N; i++) {
			int il = std::max(i - 1, 0), ir = std::min(i + 1, N);
			int jl = std::max(j - 1, 0), jr = std::min(j + 1, N);
			float gx = (H(ir, j) - H(il, j)) / ((float)(ir - il) * step);
			float gz = (H(i, jr) - H(i, jl)) / ((float)(jr - jl) * step);
			m.vertex(p3(-2.0f + step * i, H(i, j), -2.0f + step * j), unitv(p3(-gx, 1.0f, -gz)));
		}
	for (int j = 0; j < N; j++)
		for (int i = 0; i < N; i++) {
			uint32_t patch = (uint32_t)((j * 8 / N) * 8 + i * 8 / N);
			uint32_t mt = palette[patch * 7 % 64];
			uint32_t a = first + (uint32_t)(j * (N + 1) + i);
			uint32_t b = a + 1, c = a + (uint32_t)(N + 1), d = c + 1;
			m.tri(a, c, d, mt);
			m.tri(a, d, b, mt);
		}
	std::vector<P3> sv;
	std::vector<uint32_t> sf;
	unit_icosphere(sv, sf);
	for (int k = 0; k < spheres; k++) {
		float x = s.range(-1.9f, 1.9f);
		float z = s.range(-1.9f, 1.9f);
		float r = s.range(0.02f, 0.1f);
		float lift = s.range(0.2f, 1.0f);
		float y = height((x + 2.0f) * 0.25f, (z + 2.0f) * 0.25f) + r * lift;
		uint32_t mt = palette[(uint32_t)(s.bits() % 64)];
		uint32_t base = (uint32_t)(m.pos.size() / 3);
		for (const P3 &u : sv)
			m.vertex(add(p3(x, y, z), scale(u, r)), u);
		for (size_t t = 0; t < sf.size(); t += 3)
			m.tri(base + sf[t], base + sf[t + 1], base + sf[t + 2], mt);
	}
	int cols = 1;
	while (cols * cols < emitters)
		cols++;
	int rows = (emitters + cols - 1) / cols;
	float cx = 3.6f / cols, cz = 3.6f / rows;
	float size = std::min(cx, cz) * 0.4f;
	for (int k = 0; k < emitters; k++) {
		float x0 = -1.8f + cx * (k % cols) + (cx - size) * 0.5f;
		float z0 = -1.8f + cz * (k / cols) + (cz - size) * 0.5f;
		float radiance = log_radiance ? 0.1f * exp_halving(s.range(0.0f, 6.90775528f)) : s.range(1.0f, 10.0f);
		uint32_t mt = m.light(radiance);
		P3 a = p3(x0, 1.2f, z0), b = p3(x0 + size, 1.2f, z0), c = p3(x0 + size, 1.2f, z0 + size),
		   d = p3(x0, 1.2f, z0 + size);
		m.facet(a, b, c, mt);
		m.facet(a, c, d, mt);
	}
	m.camera(0, 1.0f, 2.4f, 0, -0.3f, 0);
}

/* ------------------------------------------------------------ SAH build -- */

struct Box {
	float lo[3], hi[3];
};

/* glm::min / glm::max: (y < x) ? y : x */
inline float lesser(float a, float b) { return b < a ? b : a; }
inline float greater(float a, float b) { return a < b ? b : a; }

inline void grow(Box &dst, const Box &b)
{
	for (int k = 0; k < 3; k++) {
		dst.lo[k] = lesser(dst.lo[k], b.lo[k]);
		dst.hi[k] = greater(dst.hi[k], b.hi[k]);
	}
}

inline Box empty_box()
{
	Box b;
	for (int k = 0; k < 3; k++) {
		b.lo[k] = FLT_MAX;
		b.hi[k] = -FLT_MAX;
	}
	return b;
}

/* BoundingBox::surface_area (include/bbox.hpp:14-25) */
inline float area(const Box &b)
{
	float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
	return 2.0f * (dx * dy + dy * dz + dx * dz);
}

struct SahNode {
	Box box;
	int32_t kid[2] = {-1, -1};
	uint32_t first = 0, count = 0; /* a leaf when count > 0 */
};

struct SahTree {
	std::vector<SahNode> node;
	std::vector<uint32_t> order; /* primitive ids in leaf order */
};

/* Top-down binned SAH: 32 bins over the centroid range of each axis, cost
 * 1 + (nL * A_L + nR * A_R) / A; a node of at most max_leaf primitives stays
 * a leaf unless a split costs less than its primitive count.  The partition
 * is stable, so each child keeps its parent's primitive order. */
void sah_build(const std::vector<Box> &boxes, int max_leaf, SahTree &t)
{
	const int BINS = 32;
	size_t n = boxes.size();
	t.node.clear();
	t.order.resize(n);
	if (!n)
		return;
	std::vector<float> mid(3 * n);
	for (size_t i = 0; i < n; i++) {
		t.order[i] = (uint32_t)i;
		for (int k = 0; k < 3; k++)
			mid[3 * i + k] = (boxes[i].lo[k] + boxes[i].hi[k]) * 0.5f;
	}
	struct Job {
		int32_t id;
		uint32_t lo, hi;
	};
	std::vector<Job> jobs(1, Job{0, 0, (uint32_t)n});
	t.node.emplace_back();
	while (!jobs.empty()) {
		Job job = jobs.back();
		jobs.pop_back();
		Box bounds = empty_box();
		float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
		for (uint32_t i = job.lo; i < job.hi; i++) {
			uint32_t p = t.order[i];
			grow(bounds, boxes[p]);
			for (int k = 0; k < 3; k++) {
				cmin[k] = std::min(cmin[k], mid[3 * p + k]);
				cmax[k] = std::max(cmax[k], mid[3 * p + k]);
			}
		}
		t.node[job.id].box = bounds;
		uint32_t cnt = job.hi - job.lo;
		if (cnt <= 1) {
			t.node[job.id].first = job.lo;
			t.node[job.id].count = cnt;
			continue;
		}
		float parent_area = area(bounds);
		float best = FLT_MAX;
		int best_axis = -1, best_bin = 0;
		for (int a = 0; a < 3; a++) {
			float extent = cmax[a] - cmin[a];
			if (!(extent > 0.0f))
				continue;
			float per = BINS / extent;
			Box bin_box[BINS];
			uint32_t bin_n[BINS];
			for (int b = 0; b < BINS; b++) {
				bin_box[b] = empty_box();
				bin_n[b] = 0;
			}
			for (uint32_t i = job.lo; i < job.hi; i++) {
				uint32_t p = t.order[i];
				int b = std::min(std::max((int)((mid[3 * p + a] - cmin[a]) * per), 0), BINS - 1);
				bin_n[b]++;
				grow(bin_box[b], boxes[p]);
			}
			/* suffix sweep: right side of each split plane */
			float right_area[BINS];
			uint32_t right_n[BINS];
			Box acc = empty_box();
			uint32_t c = 0;
			for (int b = BINS - 1; b > 0; b--) {
				c += bin_n[b];
				for (int k = 0; k < 3; k++) {
					acc.lo[k] = std::min(acc.lo[k], bin_box[b].lo[k]);
					acc.hi[k] = std::max(acc.hi[k], bin_box[b].hi[k]);
				}
				right_n[b] = c;
				right_area[b] = c ? area(acc) : 0.0f;
			}
			/* prefix sweep: left side, and the cost of each plane */
			acc = empty_box();
			c = 0;
			for (int b = 1; b < BINS; b++) {
				c += bin_n[b - 1];
				for (int k = 0; k < 3; k++) {
					acc.lo[k] = std::min(acc.lo[k], bin_box[b - 1].lo[k]);
					acc.hi[k] = std::max(acc.hi[k], bin_box[b - 1].hi[k]);
				}
				if (!c || !right_n[b])
					continue;
				float cost = 1.0f + ((float)c * area(acc) + (float)right_n[b] * right_area[b]) / parent_area;
				if (cost < best) {
					best = cost;
					best_axis = a;
					best_bin = b;
				}
			}
		}
		if ((int)cnt <= max_leaf && (best_axis < 0 || (float)cnt <= best)) {
			t.node[job.id].first = job.lo;
			t.node[job.id].count = cnt;
			continue;
		}
		uint32_t split = job.lo + cnt / 2; /* all centroids equal: halve by index */
		if (best_axis >= 0) {
			float per = BINS / (cmax[best_axis] - cmin[best_axis]);
			float origin = cmin[best_axis];
			std::vector<uint32_t> left, right;
			for (uint32_t i = job.lo; i < job.hi; i++) {
				uint32_t p = t.order[i];
				int b = std::min(std::max((int)((mid[3 * p + best_axis] - origin) * per), 0), BINS - 1);
				(b < best_bin ? left : right).push_back(p);
			}
			std::copy(left.begin(), left.end(), t.order.begin() + job.lo);
			std::copy(right.begin(), right.end(), t.order.begin() + job.lo + left.size());
			split = job.lo + (uint32_t)left.size();
			if (split == job.lo || split == job.hi)
				split = job.lo + cnt / 2;
		}
		int32_t l = (int32_t)t.node.size();
		t.node.emplace_back();
		t.node.emplace_back();
		t.node[job.id].kid[0] = l;
		t.node[job.id].kid[1] = l + 1;
		jobs.push_back(Job{l + 1, split, job.hi});
		jobs.push_back(Job{l, job.lo, split});
	}
}

inline float as_float(int32_t i)
{
	float f;
	memcpy(&f, &i, 4);
	return f;
}

/* serialize() of source/bvh.cpp:213-260 over the SAH tree: a pre-order walk
 * writing {leaf, object, hit, miss}, min, max per record; hit is the next
 * record, miss the record after this subtree (or the parent's miss). */
struct Threader {
	const SahTree &t;
	const std::vector<Box> &boxes;
	std::vector<uint32_t> records; /* records of each subtree */
	std::vector<float> out;

	Threader(const SahTree &tree, const std::vector<Box> &b) : t(tree), boxes(b), records(tree.node.size(), 0)
	{
		/* children have larger ids than their parent: count bottom-up */
		for (size_t i = t.node.size(); i-- > 0;) {
			const SahNode &nd = t.node[i];
			records[i] = nd.count ? nd.count : 1 + records[nd.kid[0]] + records[nd.kid[1]];
		}
	}
	void record(float leaf, int32_t object, int32_t hit, int32_t miss, const Box &b)
	{
		const float r[12] = {leaf, as_float(object), as_float(hit), as_float(miss), b.lo[0], b.lo[1], b.lo[2], 0.0f,
			b.hi[0], b.hi[1], b.hi[2], 0.0f};
		out.insert(out.end(), r, r + 12);
	}
	void write(int32_t i, int32_t miss)
	{
		const SahNode &nd = t.node[i];
		int32_t here = (int32_t)(out.size() / 4);
		if (nd.count) {
			for (uint32_t k = 0; k < nd.count; k++) {
				uint32_t prim = t.order[nd.first + k];
				int32_t next = k + 1 < nd.count ? here + 3 * (int32_t)(k + 1) : miss;
				record(1.0f, (int32_t)prim, next, next, boxes[prim]);
			}
			return;
		}
		int32_t left = here + 3;
		int32_t right = left + 3 * (int32_t)records[nd.kid[0]];
		record(0.0f, -1, left, miss, nd.box);
		write(nd.kid[0], right);
		write(nd.kid[1], miss);
	}
};

} /* namespace */

struct oracle_generated {
	Mesh m;
};

extern "C" {

int oracle_generate_scene(const char *name, uint64_t seed, oracle_generated **out)
{
	if (!name || !out)
		return -1;
	std::string n(name);
	oracle_generated *g = new oracle_generated();
	if (n == "box4k")
		box_scene(g->m, seed, 4096);
	else if (n == "box64")
		box_scene(g->m, seed, 64);
	else if (n == "terrain")
		terrain_scene(g->m, seed, 512, 2000, 512, false);
	else if (n == "terrain_s")
		terrain_scene(g->m, seed, 256, 400, 512, false);
	else if (n == "terrain_m")
		terrain_scene(g->m, seed, 512, 1500, 512, false);
	else if (n == "terrain_l")
		terrain_scene(g->m, seed, 1024, 6000, 32768, true);
	else {
		delete g;
		return -1;
	}
	*out = g;
	return 0;
}

void oracle_generated_view(const oracle_generated *g, oracle_scene_arrays *v)
{
	v->positions = g->m.pos.data();
	v->normals = g->m.nrm.data();
	v->indices = g->m.idx.data();
	v->material_indices = g->m.mat.data();
	v->materials = g->m.mats.data();
	v->vertex_count = (uint32_t)(g->m.pos.size() / 3);
	v->triangle_count = (uint32_t)g->m.mat.size();
	v->material_count = (uint32_t)g->m.mats.size();
	memcpy(v->eye, g->m.eye, 12);
	memcpy(v->target, g->m.target, 12);
	v->fov_deg = g->m.fov;
}

void oracle_generated_destroy(oracle_generated *g) { delete g; }

int64_t oracle_build_sah(const float *positions, const uint32_t *indices, uint32_t triangle_count, int max_leaf,
		float *out_vec4, uint64_t capacity)
{
	std::vector<Box> boxes(triangle_count);
	for (uint32_t i = 0; i < triangle_count; i++) {
		const float *a = positions + 3 * (size_t)indices[3 * i];
		const float *b = positions + 3 * (size_t)indices[3 * i + 1];
		const float *c = positions + 3 * (size_t)indices[3 * i + 2];
		/* Submesh::bvh (include/mesh.hpp:48-78): min(p1, min(p2, p3)); the
		 * builder sees every zero as +0 so its mins and maxes are functions
		 * of the values alone */
		for (int k = 0; k < 3; k++) {
			boxes[i].lo[k] = lesser(a[k], lesser(b[k], c[k])) + 0.0f;
			boxes[i].hi[k] = greater(a[k], greater(b[k], c[k])) + 0.0f;
		}
	}
	SahTree t;
	sah_build(boxes, max_leaf < 1 ? 4 : max_leaf, t);
	if (t.node.empty())
		return 0;
	/* leaf records carry the primitive's own box as Submesh::bvh made it
	 * (with its signed zeros) */
	for (uint32_t i = 0; i < triangle_count; i++) {
		const float *a = positions + 3 * (size_t)indices[3 * i];
		const float *b = positions + 3 * (size_t)indices[3 * i + 1];
		const float *c = positions + 3 * (size_t)indices[3 * i + 2];
		for (int k = 0; k < 3; k++) {
			boxes[i].lo[k] = lesser(a[k], lesser(b[k], c[k]));
			boxes[i].hi[k] = greater(a[k], greater(b[k], c[k]));
		}
	}
	Threader th(t, boxes);
	th.write(0, -1);
	uint64_t count = th.out.size() / 4;
	if (out_vec4) {
		if (count > capacity)
			return -1;
		memcpy(out_vec4, th.out.data(), th.out.size() * sizeof(float));
	}
	return (int64_t)count;
}

uint32_t oracle_scene_lights(const float *positions, const uint32_t *indices, const uint32_t *material_indices,
		uint32_t triangle_count, const kgr_material *materials, kgr_triangle_light *out)
{
	uint32_t n = 0;
	for (uint32_t i = 0; i < triangle_count; i++) {
		const kgr_material &m = materials[material_indices ? material_indices[i] : 0];
		if (!(m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f))
			continue;
		if (out) {
			const float *a = positions + 3 * (size_t)indices[3 * i];
			const float *b = positions + 3 * (size_t)indices[3 * i + 1];
			const float *c = positions + 3 * (size_t)indices[3 * i + 2];
			kgr_triangle_light &l = out[n];
			for (int k = 0; k < 3; k++) {
				l.a[k] = a[k];
				l.ab[k] = b[k] - a[k];
				l.ac[k] = c[k] - a[k];
				l.intensity[k] = m.emission[k];
			}
		}
		n++;
	}
	return n;
}

void oracle_camera(const float eye[3], const float target[3], const float up[3], float fov_deg, float aspect,
		float center[3], float ax_u[3], float ax_v[3], float ax_w[3])
{
	/* uvw_frame, include/camera.hpp:45-63: w = lookat - eye; u = normalize(
	 * cross(w, up)); v = normalize(cross(u, w)); |v| = |w| tan(fov / 2);
	 * |u| = |v| aspect */
	P3 e = p3(eye[0], eye[1], eye[2]);
	P3 w = sub(p3(target[0], target[1], target[2]), e);
	P3 upv = p3(up[0], up[1], up[2]);
	float wlen = sqrtf(dotp(w, w));
	/* glm::cross(x, y) = x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y */
	auto glm_cross = [](P3 x, P3 y) {
		return p3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
	};
	P3 u = unitv(glm_cross(w, upv));
	P3 v = unitv(glm_cross(u, w));
	float half = fov_deg * (float)0.01745329251994329576923690768489 / 2.0f; /* glm::radians(fov) / 2 */
	float vlen = wlen * tanf(half);
	v = scale(v, vlen);
	u = scale(u, vlen * aspect);
	memcpy(center, eye, 12);
	ax_u[0] = u.x; ax_u[1] = u.y; ax_u[2] = u.z;
	ax_v[0] = v.x; ax_v[1] = v.y; ax_v[2] = v.z;
	ax_w[0] = w.x; ax_w[1] = w.y; ax_w[2] = w.z;
}

} /* extern "C" */
