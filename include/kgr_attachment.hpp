/*
 * kgr_attachment.hpp -- header-only C++ view of the kgr C ABI with the
 * member functions of the reference's AttachmentRTX
 * (include/amadeus/armada.cuh:107-139): attach, load, unload, set_option,
 * get_option (std::variant<int, float, bool, std::string>) and render.
 *
 * The reference's own types (glm, vk::Extent2D, OptixTraversableHandle,
 * HitRecord) are not needed here: the extent is {width, height}, the launch
 * information is kgr_launch_info (ArmadaLaunchInfo with POD fields), and the
 * acceleration structure is a kgr_scene.  Failures throw kgr::Error, as the
 * reference's CUDA_CHECK/OPTIX_CHECK throw; the C ABI below never does.
 */
#ifndef KGR_ATTACHMENT_HPP_
#define KGR_ATTACHMENT_HPP_

#include <stdexcept>
#include <string>
#include <variant>

#include "kgr.h"

namespace kgr {

struct Error : std::runtime_error {
	kgr_status status;
	Error(kgr_status s, const char *what) : std::runtime_error(what), status(s) {}
};

inline void check(kgr_status s)
{
	if (s != KGR_OK)
		throw Error(s, kgr_last_error());
}

struct Extent2D {
	uint32_t width, height;
};

class Attachment {
	kgr_attachment *m_att = nullptr;

public:
	using OptionValue = std::variant<int, float, bool, std::string>;

	explicit Attachment(const char *kind) { check(kgr_create(kind, &m_att)); }
	explicit Attachment(kgr_attachment *adopt) : m_att(adopt) {}
	Attachment(const Attachment &) = delete;
	Attachment &operator=(const Attachment &) = delete;
	~Attachment() { kgr_destroy(m_att); }

	kgr_attachment *handle() const { return m_att; }

	/* AttachmentRTX::attach(const ArmadaRTX &) learns the extent */
	void attach(Extent2D extent, int device = -1)
	{
		kgr_context ctx = {extent.width, extent.height, device, 0};
		check(kgr_attach(m_att, &ctx));
	}
	void load() { check(kgr_load(m_att)); }
	void unload() { check(kgr_unload(m_att)); }

	void set_option(const std::string &field, const OptionValue &value)
	{
		kgr_value v = {};
		if (auto p = std::get_if<int>(&value)) {
			v.tag = KGR_VALUE_INT;
			v.i = *p;
		} else if (auto f = std::get_if<float>(&value)) {
			v.tag = KGR_VALUE_FLOAT;
			v.f = *f;
		} else if (auto b = std::get_if<bool>(&value)) {
			v.tag = KGR_VALUE_BOOL;
			v.b = *b;
		} else {
			v.tag = KGR_VALUE_STRING;
			v.s = std::get<std::string>(value).c_str();
		}
		check(kgr_set_option(m_att, field.c_str(), &v));
	}

	OptionValue get_option(const std::string &field) const
	{
		kgr_value v = {};
		check(kgr_get_option(m_att, field.c_str(), &v));
		switch (v.tag) {
		case KGR_VALUE_FLOAT: return v.f;
		case KGR_VALUE_BOOL: return v.b != 0;
		case KGR_VALUE_STRING: return std::string(v.s ? v.s : "");
		default: return v.i;
		}
	}

	/* AttachmentRTX::render(const ArmadaRTX *, const ArmadaLaunchInfo &,
	 * optional<handle>, vector<HitRecord> *, const vk::Extent2D &) */
	void render(const kgr_launch_info &info, const kgr_scene *scene, void *stream = nullptr)
	{
		check(kgr_render(m_att, &info, scene, stream));
	}
};

} /* namespace kgr */

#endif
