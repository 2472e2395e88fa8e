#pragma once
#include "../glm_shim.hpp"
