/* stand-in: everything the builder needs is in glm/glm.hpp (TEST INFRASTRUCTURE) */
#pragma once
#include "../glm.hpp"
