// Test infrastructure only: entry header of the vector-math subset (shim_core.hpp).
#pragma once
#include "shim_core.hpp"
