// Project-written stream state for the reference's tree serialisation.
//
// openvdb::Grid and the tree templates call a few stream-state accessors
// that live in the reference's io/Archive.cc, which needs Boost and is not
// built here.  The accessors the node (de)serialisers use (format version,
// data compression, background pointer) are given working definitions on
// std::ios_base::iword/pword slots of our own, so the test oracle can write
// and read a tree with the reference's own RootNode / InternalNode /
// LeafNode / io::writeCompressedValues code.  No StreamMetadata object is
// ever attached (getStreamMetadataPtr returns null: not seekable, no delayed
// loading); the StreamMetadata members below only satisfy the linker.
#include <openvdb/Exceptions.h>
#include <openvdb/io/DelayedLoadMetadata.h>
#include <openvdb/io/io.h>
#include <openvdb/version.h>

namespace openvdb {
OPENVDB_USE_VERSION_NAMESPACE
namespace OPENVDB_VERSION_NAME {
namespace io {

namespace {

[[noreturn]] void noIo() { OPENVDB_THROW(IoError, "stream metadata is not built into the test oracle"); }

struct Slots {
    int fileVersion = std::ios_base::xalloc();
    int libMajor = std::ios_base::xalloc();
    int libMinor = std::ios_base::xalloc();
    int compression = std::ios_base::xalloc();
    int background = std::ios_base::xalloc();
    int gridClass = std::ios_base::xalloc();
    int halfFloat = std::ios_base::xalloc();
    int gridStats = std::ios_base::xalloc();
};

Slots& slots() {
    static Slots s;
    return s;
}

}  // namespace

bool StreamMetadata::seekable() const { noIo(); }
bool StreamMetadata::delayedLoadMeta() const { noIo(); }
void StreamMetadata::setLeaf(uint64_t) { noIo(); }
uint64_t StreamMetadata::leaf() const { noIo(); }
MetaMap& StreamMetadata::gridMetadata() { noIo(); }
const MetaMap& StreamMetadata::gridMetadata() const { noIo(); }
DelayedLoadMetadata::MaskType DelayedLoadMetadata::getMask(size_t) const { noIo(); }
DelayedLoadMetadata::CompressedSizeType DelayedLoadMetadata::getCompressedSize(size_t) const { noIo(); }

uint32_t getFormatVersion(std::ios_base& s) { return uint32_t(s.iword(slots().fileVersion)); }
void checkFormatVersion(std::ios_base& s) {
    if (getFormatVersion(s) == 0) OPENVDB_THROW(IoError, "stream has no file format version");
}
VersionId getLibraryVersion(std::ios_base& s) {
    return VersionId(uint32_t(s.iword(slots().libMajor)), uint32_t(s.iword(slots().libMinor)));
}
void setVersion(std::ios_base& s, const VersionId& lib, uint32_t fileVersion) {
    s.iword(slots().fileVersion) = long(fileVersion);
    s.iword(slots().libMajor) = long(lib.first);
    s.iword(slots().libMinor) = long(lib.second);
}
uint32_t getDataCompression(std::ios_base& s) { return uint32_t(s.iword(slots().compression)); }
void setDataCompression(std::ios_base& s, uint32_t c) { s.iword(slots().compression) = long(c); }
uint32_t getGridClass(std::ios_base& s) { return uint32_t(s.iword(slots().gridClass)); }
void setGridClass(std::ios_base& s, uint32_t c) { s.iword(slots().gridClass) = long(c); }
bool getHalfFloat(std::ios_base& s) { return s.iword(slots().halfFloat) != 0; }
void setHalfFloat(std::ios_base& s, bool b) { s.iword(slots().halfFloat) = b ? 1 : 0; }
bool getWriteGridStatsMetadata(std::ios_base& s) { return s.iword(slots().gridStats) != 0; }
void setWriteGridStatsMetadata(std::ios_base& s, bool b) { s.iword(slots().gridStats) = b ? 1 : 0; }
const void* getGridBackgroundValuePtr(std::ios_base& s) { return s.pword(slots().background); }
void setGridBackgroundValuePtr(std::ios_base& s, const void* bg) {
    s.pword(slots().background) = const_cast<void*>(bg);
}
SharedPtr<StreamMetadata> getStreamMetadataPtr(std::ios_base&) { return SharedPtr<StreamMetadata>(); }

}  // namespace io
}  // namespace OPENVDB_VERSION_NAME
}  // namespace openvdb
