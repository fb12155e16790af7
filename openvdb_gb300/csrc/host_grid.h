// The library-owned host level set (gbls_host_grid in gbls.h), shared by
// the fixture builders and the .vdb file reader: one OpenVDB FloatGrid
// narrow band in the exchange layout (tree order, 0 at child slots of the
// tile tables), handed out through gbls_host_grid_view.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gbls.h"

struct gbls_host_grid {
    double voxel_size = 1.0;
    double translation[3] = {0.0, 0.0, 0.0};
    int32_t map_type = GBLS_MAP_UNIFORM_SCALE;
    float background = 3.0f;
    std::vector<int32_t> leaf_origins;
    std::vector<uint64_t> leaf_masks;
    std::vector<float> leaf_values;
    std::vector<int32_t> lower_origins;
    std::vector<float> lower_tiles;
    std::vector<int32_t> upper_origins;
    std::vector<float> upper_tiles;
    std::vector<int32_t> root_tile_origins;
    std::vector<float> root_tile_values;
};

namespace gbls_host {
// Sets the message gbls_host_last_error returns (per thread).
void set_error(const std::string& msg);
}  // namespace gbls_host
