// Test infrastructure only: entry header of the vector-math subset (shim_core.hpp, shim_geometry.hpp).
#pragma once
#include "shim_core.hpp"
#include "shim_geometry.hpp"
