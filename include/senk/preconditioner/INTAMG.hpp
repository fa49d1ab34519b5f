// The reference header of the same path (Library/preconditioner/INTAMG.hpp) maps to the GPU facade.
#pragma once
#include "senk_gb300.hpp"
