// Project-written link stubs for the reference's file-I/O entry points.
//
// openvdb::Grid and the tree templates reference stream (de)serialisation
// symbols that live in the reference's io/Archive.cc, which needs Boost.
// Nothing on the advection path reads or writes files, so these definitions
// only satisfy the linker for the test oracle; calling any of them throws.
#include <openvdb/Exceptions.h>
#include <openvdb/io/DelayedLoadMetadata.h>
#include <openvdb/io/io.h>

namespace openvdb {
OPENVDB_USE_VERSION_NAMESPACE
namespace OPENVDB_VERSION_NAME {
namespace io {

[[noreturn]] static void noIo() { OPENVDB_THROW(IoError, "file I/O is not built into the test oracle"); }

bool StreamMetadata::seekable() const { noIo(); }
bool StreamMetadata::delayedLoadMeta() const { noIo(); }
void StreamMetadata::setLeaf(uint64_t) { noIo(); }
uint64_t StreamMetadata::leaf() const { noIo(); }
MetaMap& StreamMetadata::gridMetadata() { noIo(); }
const MetaMap& StreamMetadata::gridMetadata() const { noIo(); }
uint32_t getFormatVersion(std::ios_base&) { noIo(); }
void checkFormatVersion(std::ios_base&) { noIo(); }
uint32_t getDataCompression(std::ios_base&) { noIo(); }
const void* getGridBackgroundValuePtr(std::ios_base&) { noIo(); }
void setGridBackgroundValuePtr(std::ios_base&, const void*) { noIo(); }
SharedPtr<StreamMetadata> getStreamMetadataPtr(std::ios_base&) { noIo(); }
DelayedLoadMetadata::MaskType DelayedLoadMetadata::getMask(size_t) const { noIo(); }
DelayedLoadMetadata::CompressedSizeType DelayedLoadMetadata::getCompressedSize(size_t) const { noIo(); }

} // namespace io
} // namespace OPENVDB_VERSION_NAME
} // namespace openvdb
