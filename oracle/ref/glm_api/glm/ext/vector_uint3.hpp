// glm API header used by the reference: forwards to the restatement in glm_api.hpp (test infrastructure).
#pragma once
#include "../glm_api.hpp"
