// Host samplers for GBLS_FIELD_HOST_SAMPLED fields.
//
// gbls_host_sample_enright is a gbls_host_sample_fn evaluating the
// reference's EnrightField<float> (tools/VelocityFields.h:101-141) at each
// active voxel the way Advect::sample<false> does (tools/LevelSetAdvect.h:
// 476-493): the voxel's world position from the level set's map (index x
// scale + translation, in double), then the field at that position.  The
// field's transform is the identity transform, which is never equal to a
// level set's uniform-scale map, so the reference always takes this path.
#include <cstdint>

#include "../../include/gbls.h"
#include "../../include/gbls_fields.h"

extern "C" void gbls_host_sample_enright(void* user, int64_t n, const int32_t* ijk, float t, float* velocity) {
    const gbls_host_map* m = static_cast<const gbls_host_map*>(user);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t* q = ijk + 3 * i;
        const double x = double(q[0]) * m->scale + m->translation[0];
        const double y = double(q[1]) * m->scale + m->translation[1];
        const double z = double(q[2]) * m->scale + m->translation[2];
        gbls_enright(x, y, z, t, velocity + 3 * i);
    }
}
