// The reference's own OpenVDB -> NanoVDB conversion, for the test oracle:
// nanovdb::tools::createNanoGrid (nanovdb/tools/CreateNanoGrid.h) applied to
// a FloatGrid of the oracle, the NanoVDB buffer copied out.  Built without
// NANOVDB_USE_TBB, so node statistics combine serially in tree order.
#define NANOVDB_USE_OPENVDB
#include <nanovdb/tools/CreateNanoGrid.h>

#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "gbls.h"

namespace {
thread_local std::string gNanoError;
}

namespace vdbref_detail {
openvdb::FloatGrid::Ptr grid_of(void* g);
}

extern "C" {

const char* vdbref_nano_last_error() { return gNanoError.c_str(); }

// Size in bytes of createNanoGrid(grid, stats, checksum) when `out` is null,
// else the buffer itself (out_cap bytes available).
int vdbref_nano_float(void* g, const char* name, int stats, int checksum, uint8_t* out, int64_t out_cap,
                      int64_t* size) {
    try {
        // the grid itself, not a deepCopy(): copying a UniformScaleTranslateMap
        // perturbs its scale in the last bits
        openvdb::FloatGrid::Ptr grid = vdbref_detail::grid_of(g);
        grid->setName(name);
        auto handle = nanovdb::tools::createNanoGrid(*grid, nanovdb::tools::StatsMode(stats),
                                                     nanovdb::CheckMode(checksum));
        *size = int64_t(handle.bufferSize());
        if (out) {
            if (out_cap < *size) {
                gNanoError = "buffer too small";
                return GBLS_ERR_INVALID_ARGUMENT;
            }
            std::memcpy(out, handle.data(), size_t(*size));
        }
        return 0;
    } catch (const std::exception& e) {
        gNanoError = e.what();
        return GBLS_ERR_RUNTIME;
    }
}

// createNanoGrid<FloatGrid, ValueOnIndex>(grid, channels, includeStats, includeTiles).
int vdbref_nano_onindex(void* g, const char* name, int channels, int stats, int tiles, int checksum, uint8_t* out,
                        int64_t out_cap, int64_t* size) {
    try {
        openvdb::FloatGrid::Ptr grid = vdbref_detail::grid_of(g);
        grid->setName(name);
        auto handle = nanovdb::tools::createNanoGrid<openvdb::FloatGrid, nanovdb::ValueOnIndex>(
            *grid, uint32_t(channels), stats != 0, tiles != 0);
        if (checksum != 1)
            nanovdb::tools::updateChecksum(reinterpret_cast<nanovdb::GridData*>(handle.data()),
                                           checksum == 0 ? nanovdb::CheckMode::Disable : nanovdb::CheckMode::Full);
        *size = int64_t(handle.bufferSize());
        if (out) {
            if (out_cap < *size) {
                gNanoError = "buffer too small";
                return GBLS_ERR_INVALID_ARGUMENT;
            }
            std::memcpy(out, handle.data(), size_t(*size));
        }
        return 0;
    } catch (const std::exception& e) {
        gNanoError = e.what();
        return GBLS_ERR_RUNTIME;
    }
}

}  // extern "C"
