/*
 * glm/glm.hpp stand-in for compiling the reference's include/cuda/cast.cuh
 * on the host (TEST INFRASTRUCTURE).  glm is not vendored in the reference
 * checkout; cast.cuh only names glm::vec3 (to_f3), which is all this
 * provides.  Nothing of glm's arithmetic is used by the known answers.
 */
#pragma once

namespace glm {

struct vec3 {
	float x, y, z;
};

} /* namespace glm */
