// Test infrastructure only: entry header of the vector-math subset (shim_geometry.hpp).
#pragma once
#include "../shim_geometry.hpp"
