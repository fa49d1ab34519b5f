// The reference header of the same path (Library/utils/utils.hpp) maps to the GPU facade.
#pragma once
#include "senk_gb300.hpp"
