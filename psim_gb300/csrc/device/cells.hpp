// Construction of the device cell records (engine.cu), callable from host code.
#pragma once

#include <vector>

#include "common.cuh"
#include "engine.hpp"

namespace psim::gpu {

void build_cells(const SimDesc& d, std::vector<CellF32>& c32, std::vector<CellF64>& c64, std::vector<Sub64>& subs);

}// namespace psim::gpu
