// Exercises include/kgr_attachment.hpp (the AttachmentRTX-shaped C++ view of
// the C ABI) without a GPU: create, option round trips, the reference's
// ignore-unknown-option behaviour, type errors and the plugin export.
#include <cstdio>
#include <cstring>

#include "kgr_attachment.hpp"

int main()
{
	kgr::Attachment pt("path_tracer");
	pt.set_option("russian_roulette", true);
	pt.set_option("spp", 8);
	pt.set_option("layout", std::string("threaded"));
	pt.set_option("not_an_option", 1.5f);
	bool rr = std::get<bool>(pt.get_option("russian_roulette"));
	int spp = std::get<int>(pt.get_option("spp"));
	std::string layout = std::get<std::string>(pt.get_option("layout"));
	int unknown = std::get<int>(pt.get_option("not_an_option"));
	bool type_error = false;
	try {
		pt.set_option("spp", 2.0f);
	} catch (const kgr::Error &e) {
		type_error = e.status == KGR_ERR_TYPE;
	}
	kgr_plugin_ret r = kgr_load_attachment("restir_di");
	bool plugin = r.ptr && r.name && std::strcmp(r.name, "ReSTIR") == 0;
	kgr_destroy(r.ptr);
	std::printf("%d %d %s %d %d %d\n", rr, spp, layout.c_str(), unknown, type_error, plugin);
	return (rr && spp == 8 && layout == "threaded" && unknown == 0 && type_error && plugin) ? 0 : 1;
}
