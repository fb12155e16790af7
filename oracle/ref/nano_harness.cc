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

// The reference's own ReadAccessor on a NanoVDB buffer (copied into an
// aligned HostBuffer): getValue and isActive at n index coordinates, for a
// NanoGrid<float> (fvals) or a NanoGrid<ValueOnIndex> (ivals, the
// LeafData<ValueOnIndex>::getValue decode of nanovdb/NanoVDB.h:4144-4170).
int vdbref_nano_probe(const uint8_t* buf, int64_t size, const int32_t* ijk, int64_t n, float* fvals, uint64_t* ivals,
                      uint8_t* active) {
    try {
        nanovdb::HostBuffer hb = nanovdb::HostBuffer::create(uint64_t(size));
        std::memcpy(hb.data(), buf, size_t(size));
        nanovdb::GridHandle<nanovdb::HostBuffer> handle(std::move(hb));
        if (auto* g = handle.grid<float>()) {
            auto acc = g->getAccessor();
            for (int64_t i = 0; i < n; ++i) {
                const nanovdb::Coord c(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
                fvals[i] = acc.getValue(c);
                active[i] = acc.isActive(c) ? 1 : 0;
            }
            return 0;
        }
        if (auto* g = handle.grid<nanovdb::ValueOnIndex>()) {
            auto acc = g->getAccessor();
            for (int64_t i = 0; i < n; ++i) {
                const nanovdb::Coord c(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
                ivals[i] = acc.getValue(c);
                active[i] = acc.isActive(c) ? 1 : 0;
            }
            return 0;
        }
        gNanoError = "neither a NanoGrid<float> nor a NanoGrid<ValueOnIndex>";
        return GBLS_ERR_UNSUPPORTED;
    } catch (const std::exception& e) {
        gNanoError = e.what();
        return GBLS_ERR_RUNTIME;
    }
}

}  // extern "C"
