/* stand-in: what the programs need is in glm/glm.hpp (TEST INFRASTRUCTURE) */
#pragma once
#include "../glm.hpp"
