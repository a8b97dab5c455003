/*
 * project.cpp -- reading a Kobra project from disk (kgr_project_*).
 *
 * The on-disk project is what Project::save writes (source/project.cpp:
 * 63-205) and Project::load_project / load_scene read
 * (include/project.hpp:58-92, source/project.cpp:242-560):
 *
 *   <dir>/project.den            "@scenes N" then N scene file names
 *   <dir>/<scene>.kobra          text: "@entity <name>" starts an element;
 *                                ".transform px py pz rx ry rz sx sy sz",
 *                                ".mesh K" followed by K lines
 *                                "<submesh file>, <material file>",
 *                                ".renderable", ".camera <fov> <aspect>";
 *                                '#' comments; "@materials" + ".list K"
 *   <dir>/.cache/<submesh file>  int32 vertex count, int32 index count,
 *                                Vertex[] (include/vertex.hpp:15-20: position,
 *                                normal, uv, tangent, bitangent = 56 bytes),
 *                                uint32 indices[]  (the mesh cache)
 *   <dir>/assets/<material file> "name: ...", "diffuse: r,g,b", "specular:",
 *                                "emission:", "roughness:", "refraction:",
 *                                "type:", three texture lines
 *                                (source/daemons/material.cpp:37-97)
 *
 * An entity's model matrix is Transform::matrix() (include/transform.hpp:
 * 67-72): translate(position) * mat4_cast(quat(radians(rotation))) *
 * scale(scale).  glm is not in the reference checkout; its published
 * scalar formulas are restated below (quaternion from Euler angles,
 * quaternion to matrix, matrix product summed column by column in order).
 * A camera entity's frame follows uvw_frame (include/camera.hpp:45-63) with
 * Transform::forward()/up() (transform.hpp:98-112), which build the
 * quaternion from the rotation in degrees without converting it to radians;
 * that is kept, so a saved camera looks where the reference's looks.
 *
 * Only entities marked renderable contribute geometry, as only Renderable
 * components reach ArmadaRTX.  Materials are shared by name, as the
 * material daemon does.  A missing submesh file is skipped, as the
 * reference skips it; a missing material file is an error (the reference
 * would index its material list with -1).  Texture names are kept but not
 * sampled.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "kgr_internal.h"

namespace kgr {

namespace {

/* ------------------------------------------------------------- glm math -- */

struct V3 {
	float x, y, z;
};

/* column-major, m[c][r] as glm::mat4 */
struct M4 {
	float m[4][4];
};

M4 identity4()
{
	M4 r;
	memset(&r, 0, sizeof(r));
	for (int i = 0; i < 4; i++)
		r.m[i][i] = 1.0f;
	return r;
}

/* glm operator*(mat4, mat4): column i = sum over k of a[k] * b[i][k] */
M4 mul4(const M4 &a, const M4 &b)
{
	M4 r;
	for (int i = 0; i < 4; i++)
		for (int row = 0; row < 4; row++)
			r.m[i][row] = a.m[0][row] * b.m[i][0] + a.m[1][row] * b.m[i][1] + a.m[2][row] * b.m[i][2]
				+ a.m[3][row] * b.m[i][3];
	return r;
}

/* glm::translate(m, v): column 3 = m[0] v.x + m[1] v.y + m[2] v.z + m[3] */
M4 translate4(const M4 &m, V3 v)
{
	M4 r = m;
	for (int row = 0; row < 4; row++)
		r.m[3][row] = m.m[0][row] * v.x + m.m[1][row] * v.y + m.m[2][row] * v.z + m.m[3][row];
	return r;
}

/* glm::scale(m, v) */
M4 scale4(const M4 &m, V3 v)
{
	M4 r = m;
	for (int row = 0; row < 4; row++) {
		r.m[0][row] = m.m[0][row] * v.x;
		r.m[1][row] = m.m[1][row] * v.y;
		r.m[2][row] = m.m[2][row] * v.z;
	}
	return r;
}

struct Quat {
	float w, x, y, z;
};

/* glm::quat(vec3 euler): half-angle cosines and sines per axis */
Quat quat_from_euler(V3 e)
{
	float cx = cosf(e.x * 0.5f), cy = cosf(e.y * 0.5f), cz = cosf(e.z * 0.5f);
	float sx = sinf(e.x * 0.5f), sy = sinf(e.y * 0.5f), sz = sinf(e.z * 0.5f);
	Quat q;
	q.w = cx * cy * cz + sx * sy * sz;
	q.x = sx * cy * cz - cx * sy * sz;
	q.y = cx * sy * cz + sx * cy * sz;
	q.z = cx * cy * sz - sx * sy * cz;
	return q;
}

/* glm::mat4_cast(q) */
M4 mat4_cast(Quat q)
{
	float qxx = q.x * q.x, qyy = q.y * q.y, qzz = q.z * q.z;
	float qxz = q.x * q.z, qxy = q.x * q.y, qyz = q.y * q.z;
	float qwx = q.w * q.x, qwy = q.w * q.y, qwz = q.w * q.z;
	M4 r = identity4();
	r.m[0][0] = 1.0f - 2.0f * (qyy + qzz);
	r.m[0][1] = 2.0f * (qxy + qwz);
	r.m[0][2] = 2.0f * (qxz - qwy);
	r.m[1][0] = 2.0f * (qxy - qwz);
	r.m[1][1] = 1.0f - 2.0f * (qxx + qzz);
	r.m[1][2] = 2.0f * (qyz + qwx);
	r.m[2][0] = 2.0f * (qxz + qwy);
	r.m[2][1] = 2.0f * (qyz - qwx);
	r.m[2][2] = 1.0f - 2.0f * (qxx + qyy);
	return r;
}

/* glm::radians */
V3 radians3(V3 d)
{
	const float k = (float)0.01745329251994329576923690768489;
	return V3{d.x * k, d.y * k, d.z * k};
}

V3 cross3(V3 a, V3 b)
{
	return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

/* glm::normalize: v * (1 / sqrt(dot(v, v))) */
V3 normalize3(V3 v)
{
	float d = v.x * v.x + v.y * v.y + v.z * v.z;
	float inv = 1.0f / sqrtf(d);
	return V3{v.x * inv, v.y * inv, v.z * inv};
}

/* glm quat * vec3: v + ((uv * w) + uuv) * 2, uv = q.xyz x v, uuv = q.xyz x uv */
V3 rotate3(Quat q, V3 v)
{
	V3 qv{q.x, q.y, q.z};
	V3 uv = cross3(qv, v);
	V3 uuv = cross3(qv, uv);
	return V3{v.x + ((uv.x * q.w) + uuv.x) * 2.0f, v.y + ((uv.y * q.w) + uuv.y) * 2.0f,
		v.z + ((uv.z * q.w) + uuv.z) * 2.0f};
}

/* Transform::matrix() */
M4 transform_matrix(V3 position, V3 rotation_deg, V3 scale)
{
	M4 p = translate4(identity4(), position);
	M4 r = mat4_cast(quat_from_euler(radians3(rotation_deg)));
	M4 s = scale4(identity4(), scale);
	return mul4(mul4(p, r), s);
}

/* ----------------------------------------------------------- the reader -- */

std::string trim(const std::string &s)
{
	size_t a = s.find_first_not_of(" \t\r");
	if (a == std::string::npos)
		return "";
	size_t b = s.find_last_not_of(" \t\r");
	return s.substr(a, b - a + 1);
}

std::string join(const std::string &dir, const std::string &a, const std::string &b = "")
{
	std::string p = dir;
	if (!p.empty() && p.back() != '/')
		p += '/';
	p += a;
	if (!b.empty())
		p += "/" + b;
	return p;
}

bool exists(const std::string &path)
{
	std::ifstream f(path, std::ios::binary);
	return f.good();
}

/* load_material (source/daemons/material.cpp:37-97): one field per line, in
 * this order, each read with its own format */
kgr_material read_material(const std::string &path, std::string &name, bool &textured)
{
	std::ifstream f(path);
	KGR_REQUIRE(f.is_open(), KGR_ERR_INVALID_ARGUMENT, "material file missing: " + path);
	kgr_material m;
	memset(&m, 0, sizeof(m));
	/* Material's defaults (include/material.hpp:21-35) for fields a short
	 * file leaves out */
	m.diffuse[0] = 1.0f;
	m.diffuse[2] = 1.0f;
	m.roughness = 0.001f;
	m.refraction = 1.0f;
	m.type = 1 << 2; /* Shading::eDiffuse */
	char buf[1024];
	char tex[3][1024] = {{0}, {0}, {0}};
	std::string line;
	auto next = [&]() -> const char * {
		if (!std::getline(f, line))
			line.clear();
		return line.c_str();
	};
	buf[0] = 0;
	sscanf(next(), "name: %1023s", buf);
	name = buf;
	sscanf(next(), "diffuse: %f,%f,%f", &m.diffuse[0], &m.diffuse[1], &m.diffuse[2]);
	sscanf(next(), "specular: %f,%f,%f", &m.specular[0], &m.specular[1], &m.specular[2]);
	sscanf(next(), "emission: %f,%f,%f", &m.emission[0], &m.emission[1], &m.emission[2]);
	sscanf(next(), "roughness: %f", &m.roughness);
	sscanf(next(), "refraction: %f", &m.refraction);
	int type = m.type;
	sscanf(next(), "type: %d", &type);
	m.type = type;
	sscanf(next(), "albedo_texture: %1023s", tex[0]);
	sscanf(next(), "normal_texture: %1023s", tex[1]);
	sscanf(next(), "roughness_texture: %1023s", tex[2]);
	textured = tex[0][0] || tex[1][0] || tex[2][0];
	return m;
}

/* load_mesh (source/project.cpp:222-239) */
bool read_submesh(const std::string &path, std::vector<float> &pos, std::vector<float> &nrm,
		std::vector<uint32_t> &idx)
{
	std::ifstream f(path, std::ios::binary);
	if (!f.is_open())
		return false;
	int32_t nv = 0, ni = 0;
	f.read((char *)&nv, 4);
	f.read((char *)&ni, 4);
	KGR_REQUIRE(f.good() && nv >= 0 && ni >= 0 && ni % 3 == 0, KGR_ERR_INVALID_ARGUMENT,
		"malformed submesh file: " + path);
	std::vector<float> v((size_t)nv * 14);
	f.read((char *)v.data(), (std::streamsize)(v.size() * 4));
	idx.resize((size_t)ni);
	f.read((char *)idx.data(), (std::streamsize)(idx.size() * 4));
	KGR_REQUIRE(f.good() || (f.eof() && f.gcount() == (std::streamsize)(idx.size() * 4)), KGR_ERR_INVALID_ARGUMENT,
		"truncated submesh file: " + path);
	pos.resize((size_t)nv * 3);
	nrm.resize((size_t)nv * 3);
	for (int32_t i = 0; i < nv; i++) {
		memcpy(&pos[3 * (size_t)i], &v[14 * (size_t)i], 12);
		memcpy(&nrm[3 * (size_t)i], &v[14 * (size_t)i + 3], 12);
	}
	for (uint32_t k : idx)
		KGR_REQUIRE(k < (uint32_t)nv, KGR_ERR_INVALID_ARGUMENT, "index out of range in " + path);
	return true;
}

} /* namespace */

} /* namespace kgr */

using namespace kgr;

struct kgr_project {
	std::string directory;
	std::vector<std::string> scene_files;
};

struct kgr_project_scene {
	struct Entity {
		std::string name;
		float position[3] = {0, 0, 0}, rotation[3] = {0, 0, 0}, scale[3] = {1, 1, 1};
		float model[16];
		bool renderable = false, has_mesh = false, has_camera = false;
		float fov = 0.0f, aspect = 0.0f;
		uint32_t mesh_first = 0, mesh_count = 0;
	};
	std::vector<Entity> entities;
	std::vector<std::vector<float>> positions, normals;
	std::vector<std::vector<uint32_t>> indices, material_indices;
	std::vector<float> models; /* 16 per mesh */
	std::vector<kgr_mesh> meshes;
	std::vector<kgr_material> materials;
	std::vector<std::string> material_names;
	uint32_t textured_materials = 0, missing_meshes = 0;
};

extern "C" {

kgr_status kgr_transform_matrix(const float position[3], const float rotation_deg[3], const float scale[3],
		float out[16])
{
	return guard_call([&] {
		KGR_REQUIRE(position && rotation_deg && scale && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		M4 m = transform_matrix(V3{position[0], position[1], position[2]},
			V3{rotation_deg[0], rotation_deg[1], rotation_deg[2]}, V3{scale[0], scale[1], scale[2]});
		memcpy(out, m.m, 64);
	});
}

kgr_status kgr_project_open(const char *directory, kgr_project **out)
{
	return guard_call([&] {
		KGR_REQUIRE(directory && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*out = nullptr;
		std::unique_ptr<kgr_project> p(new kgr_project());
		p->directory = directory;
		std::string den = join(directory, "project.den");
		std::ifstream f(den);
		KGR_REQUIRE(f.is_open(), KGR_ERR_INVALID_ARGUMENT, "project file does not exist: " + den);
		std::string token;
		int n = -1;
		f >> token >> n;
		KGR_REQUIRE(token == "@scenes" && n >= 0, KGR_ERR_INVALID_ARGUMENT, "invalid project file: " + den);
		for (int i = 0; i < n; i++) {
			std::string s;
			KGR_REQUIRE((bool)(f >> s), KGR_ERR_INVALID_ARGUMENT, "project file lists fewer scenes than it says");
			KGR_REQUIRE(exists(join(directory, s)), KGR_ERR_INVALID_ARGUMENT, "scene file does not exist: " + s);
			p->scene_files.push_back(s);
		}
		*out = p.release();
	});
}

kgr_status kgr_project_scene_count(const kgr_project *p, uint32_t *count)
{
	return guard_call([&] {
		KGR_REQUIRE(p && count, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*count = (uint32_t)p->scene_files.size();
	});
}

kgr_status kgr_project_scene_file(const kgr_project *p, uint32_t index, const char **name)
{
	return guard_call([&] {
		KGR_REQUIRE(p && name, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(index < p->scene_files.size(), KGR_ERR_INVALID_ARGUMENT, "scene index out of range");
		*name = p->scene_files[index].c_str();
	});
}

kgr_status kgr_project_read_scene(const kgr_project *p, int32_t index, kgr_project_scene **out)
{
	return guard_call([&] {
		KGR_REQUIRE(p && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		*out = nullptr;
		if (index < 0)
			index = 0; /* default_scene_index */
		KGR_REQUIRE((size_t)index < p->scene_files.size(), KGR_ERR_INVALID_ARGUMENT, "no such scene");
		std::string path = join(p->directory, p->scene_files[index]);
		std::ifstream f(path);
		KGR_REQUIRE(f.is_open(), KGR_ERR_INVALID_ARGUMENT, "scene file does not exist: " + path);
		std::vector<std::string> lines;
		for (std::string l; std::getline(f, l);)
			lines.push_back(l);

		struct Element {
			bool entity = false;
			kgr_project_scene::Entity e;
			bool has_transform = false;
			std::vector<std::string> meshes, mats;
		};
		std::vector<Element> elements;
		Element *cur = nullptr;
		size_t i = 0;
		while (i < lines.size()) {
			const std::string &line = lines[i++];
			if (line.empty() || line[0] == '#')
				continue;
			if (line[0] == '@') {
				std::istringstream iss(line.substr(1));
				std::string type;
				iss >> type;
				if (type == "entity" || type == "materials") {
					elements.push_back(Element());
					cur = &elements.back();
					cur->entity = type == "entity";
					if (cur->entity)
						cur->e.name = trim(line.size() > 7 ? line.substr(7) : "");
				}
				continue; /* unknown element types are skipped, with their fields going to the last one */
			}
			if (line[0] != '.' || !cur)
				continue;
			std::string field = line.substr(1);
			if (field.rfind("transform", 0) == 0) {
				float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
				std::istringstream iss(field.size() > 10 ? field.substr(10) : "");
				for (int k = 0; k < 9; k++)
					iss >> v[k];
				memcpy(cur->e.position, v, 12);
				memcpy(cur->e.rotation, v + 3, 12);
				memcpy(cur->e.scale, v + 6, 12);
				cur->has_transform = true;
			} else if (field.rfind("mesh", 0) == 0) {
				int count = atoi(field.size() > 5 ? field.substr(5).c_str() : "0");
				KGR_REQUIRE(count >= 0 && i + (size_t)count <= lines.size(), KGR_ERR_INVALID_ARGUMENT,
					"mesh list runs past the end of " + path);
				cur->meshes.clear();
				cur->mats.clear();
				for (int k = 0; k < count; k++) {
					const std::string &ml = lines[i++];
					size_t a = ml.find_first_not_of(" \t");
					std::string rest = a == std::string::npos ? "" : ml.substr(a);
					size_t comma = rest.find(',');
					std::string mesh = rest.substr(0, comma);
					std::string mat;
					if (comma != std::string::npos) {
						std::istringstream iss(rest.substr(comma + 1));
						iss >> mat;
					}
					cur->meshes.push_back(mesh);
					cur->mats.push_back(mat);
				}
				cur->e.has_mesh = true;
			} else if (field.rfind("renderable", 0) == 0) {
				cur->e.renderable = true;
			} else if (field.rfind("list", 0) == 0) {
				int count = field.size() > 5 ? atoi(field.substr(5).c_str()) : 0;
				KGR_REQUIRE(count >= 0 && i + (size_t)count <= lines.size(), KGR_ERR_INVALID_ARGUMENT,
					"material list runs past the end of " + path);
				i += (size_t)count;
			} else if (field.rfind("camera", 0) == 0) {
				std::istringstream iss(field.size() > 7 ? field.substr(7) : "");
				iss >> cur->e.fov >> cur->e.aspect;
				cur->e.has_camera = true;
			}
		}

		std::unique_ptr<kgr_project_scene> sc(new kgr_project_scene());
		std::map<std::string, uint32_t> by_name;
		for (Element &el : elements) {
			if (!el.entity)
				continue;
			kgr_project_scene::Entity e = el.e;
			M4 m = transform_matrix(V3{e.position[0], e.position[1], e.position[2]},
				V3{e.rotation[0], e.rotation[1], e.rotation[2]}, V3{e.scale[0], e.scale[1], e.scale[2]});
			memcpy(e.model, m.m, 64);
			e.mesh_first = (uint32_t)sc->positions.size();
			if (e.renderable && e.has_mesh) {
				for (size_t k = 0; k < el.meshes.size(); k++) {
					std::string mname;
					bool textured = false;
					kgr_material mat = read_material(join(p->directory, "assets", el.mats[k]), mname, textured);
					uint32_t mid;
					auto it = by_name.find(mname);
					if (it != by_name.end()) {
						mid = it->second;
					} else {
						mid = (uint32_t)sc->materials.size();
						by_name[mname] = mid;
						sc->materials.push_back(mat);
						sc->material_names.push_back(mname);
						sc->textured_materials += textured ? 1 : 0;
					}
					std::vector<float> pos, nrm;
					std::vector<uint32_t> idx;
					if (!read_submesh(join(p->directory, ".cache", el.meshes[k]), pos, nrm, idx)) {
						sc->missing_meshes++;
						continue;
					}
					sc->positions.push_back(std::move(pos));
					sc->normals.push_back(std::move(nrm));
					sc->material_indices.push_back(std::vector<uint32_t>(idx.size() / 3, mid));
					sc->indices.push_back(std::move(idx));
					sc->models.insert(sc->models.end(), e.model, e.model + 16);
				}
			}
			e.mesh_count = (uint32_t)sc->positions.size() - e.mesh_first;
			sc->entities.push_back(e);
		}
		if (sc->materials.empty()) {
			/* kgr_scene_create wants one material; a scene without
			 * geometry gets the reference's default (magenta diffuse) */
			kgr_material m;
			memset(&m, 0, sizeof(m));
			m.diffuse[0] = 1.0f;
			m.diffuse[2] = 1.0f;
			m.roughness = 0.001f;
			m.refraction = 1.0f;
			m.type = 1 << 2;
			sc->materials.push_back(m);
			sc->material_names.push_back("default");
		}
		size_t n = sc->positions.size();
		sc->meshes.resize(n);
		for (size_t k = 0; k < n; k++) {
			kgr_mesh &me = sc->meshes[k];
			me.positions = sc->positions[k].data();
			me.normals = sc->normals[k].data();
			me.vertex_count = (uint32_t)(sc->positions[k].size() / 3);
			me.indices = sc->indices[k].data();
			me.material_indices = sc->material_indices[k].data();
			me.triangle_count = (uint32_t)(sc->indices[k].size() / 3);
			me.model = &sc->models[16 * k];
		}
		*out = sc.release();
	});
}

kgr_status kgr_project_scene_info_get(const kgr_project_scene *sc, kgr_project_scene_info *info)
{
	return guard_call([&] {
		KGR_REQUIRE(sc && info, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		memset(info, 0, sizeof(*info));
		info->entity_count = (uint32_t)sc->entities.size();
		info->mesh_count = (uint32_t)sc->meshes.size();
		for (const kgr_mesh &m : sc->meshes) {
			info->vertex_count += m.vertex_count;
			info->triangle_count += m.triangle_count;
		}
		info->material_count = (uint32_t)sc->materials.size();
		info->textured_materials = sc->textured_materials;
		info->missing_meshes = sc->missing_meshes;
		info->camera_entity = -1;
		for (size_t k = 0; k < sc->entities.size(); k++)
			if (sc->entities[k].has_camera) {
				info->camera_entity = (int32_t)k;
				break;
			}
	});
}

kgr_status kgr_project_scene_meshes(const kgr_project_scene *sc, const kgr_mesh **meshes, uint32_t *mesh_count,
		const kgr_material **materials, uint32_t *material_count)
{
	return guard_call([&] {
		KGR_REQUIRE(sc && meshes && mesh_count && materials && material_count, KGR_ERR_INVALID_ARGUMENT,
			"NULL argument");
		*meshes = sc->meshes.data();
		*mesh_count = (uint32_t)sc->meshes.size();
		*materials = sc->materials.data();
		*material_count = (uint32_t)sc->materials.size();
	});
}

kgr_status kgr_project_scene_entity(const kgr_project_scene *sc, uint32_t index, kgr_project_entity *out)
{
	return guard_call([&] {
		KGR_REQUIRE(sc && out, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(index < sc->entities.size(), KGR_ERR_INVALID_ARGUMENT, "entity index out of range");
		const kgr_project_scene::Entity &e = sc->entities[index];
		memset(out, 0, sizeof(*out));
		out->name = e.name.c_str();
		memcpy(out->position, e.position, 12);
		memcpy(out->rotation, e.rotation, 12);
		memcpy(out->scale, e.scale, 12);
		memcpy(out->model, e.model, 64);
		out->renderable = e.renderable;
		out->has_camera = e.has_camera;
		out->fov = e.fov;
		out->aspect = e.aspect;
		out->mesh_first = e.mesh_first;
		out->mesh_count = e.mesh_count;
	});
}

kgr_status kgr_project_scene_camera(const kgr_project_scene *sc, uint32_t entity, float aspect, kgr_launch_info *info)
{
	return guard_call([&] {
		KGR_REQUIRE(sc && info, KGR_ERR_INVALID_ARGUMENT, "NULL argument");
		KGR_REQUIRE(entity < sc->entities.size() && sc->entities[entity].has_camera, KGR_ERR_INVALID_ARGUMENT,
			"not a camera entity");
		const kgr_project_scene::Entity &e = sc->entities[entity];
		/* Transform::forward()/up(): glm::quat(rotation), the rotation taken
		 * as radians although it is stored in degrees */
		Quat q = quat_from_euler(V3{e.rotation[0], e.rotation[1], e.rotation[2]});
		V3 fwd = normalize3(rotate3(q, V3{0.0f, 0.0f, -1.0f}));
		V3 up = normalize3(rotate3(q, V3{0.0f, 1.0f, 0.0f}));
		float eye[3] = {e.position[0], e.position[1], e.position[2]};
		float target[3] = {eye[0] + fwd.x, eye[1] + fwd.y, eye[2] + fwd.z};
		float upv[3] = {up.x, up.y, up.z};
		kgr_status s = kgr_camera_setup(eye, target, upv, e.fov, aspect > 0.0f ? aspect : e.aspect, info);
		KGR_REQUIRE(s == KGR_OK, s, kgr_last_error());
	});
}

kgr_status kgr_project_scene_destroy(kgr_project_scene *sc)
{
	delete sc;
	return KGR_OK;
}

kgr_status kgr_project_close(kgr_project *p)
{
	delete p;
	return KGR_OK;
}

} /* extern "C" */
