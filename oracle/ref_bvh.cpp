/*
 * ref_bvh.cpp -- the reference's BVH builder and serialiser compiled on the
 * host, for known-answer vectors of the threaded layout.
 *
 * TEST INFRASTRUCTURE.  Compiled by oracle/Makefile (target `ref`) against
 * the reference sources where they lie (REFERENCE=<path>), into
 * oracle/_ref/ref_bvh.  It includes source/bvh.cpp (partition, serialize)
 * and through it include/bvh.hpp, bbox.hpp, transform.hpp, core.hpp,
 * vec.hpp and logger.hpp, unmodified; glm and termcolor are empty
 * submodules in the checkout, so oracle/shim_bvh stands in for them (see
 * its glm.hpp).  logger.hpp declares the log stream that KOBRA_ASSERT
 * writes to; it is defined here, as a plain stream.
 *
 * Input on stdin: uint32 n, then n boxes of 6 floats {min xyz, max xyz}.
 * Output on stdout: the buffer of serialize(partition(boxes)) as raw
 * little-endian floats (3 vec4 per node).
 */
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <limits>
#include <vector>

#include "source/bvh.cpp"

namespace kobra {
namespace detail {
std::map<void *, LogHandler> log_handlers;
}
detail::LogStream &logger(const std::string &, Log, const std::string &, bool)
{
	static detail::LogStream stream(std::cerr);
	return stream;
}
} /* namespace kobra */

int main()
{
	uint32_t n;
	if (fread(&n, 4, 1, stdin) != 1)
		return 1;
	std::vector<float> raw(6 * (size_t)n);
	if (fread(raw.data(), 4, raw.size(), stdin) != raw.size())
		return 1;
	std::vector<kobra::BoundingBox> boxes(n);
	for (uint32_t i = 0; i < n; i++) {
		const float *b = &raw[6 * (size_t)i];
		boxes[i].min = glm::vec3(b[0], b[1], b[2]);
		boxes[i].max = glm::vec3(b[3], b[4], b[5]);
	}
	std::vector<aligned_vec4> buffer;
	kobra::serialize(buffer, kobra::partition(boxes));
	for (const aligned_vec4 &v : buffer) {
		float f[4] = {v.data.x, v.data.y, v.data.z, v.data.w};
		fwrite(f, 4, 4, stdout);
	}
	return 0;
}
