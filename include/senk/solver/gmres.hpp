// The reference header of the same path (Library/solver/gmres.hpp) maps to the GPU facade.
#pragma once
#include "senk_gb300.hpp"
