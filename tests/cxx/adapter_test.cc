// Host-side checks of the C++ drop-in (include/openvdb_gb300/*.h) against
// the reference's own OpenVDB types, compiled from the reference headers:
//   1. pack(createLevelSetSphere grid) equals the library's sphere fixture
//      descriptor element for element (tree order, tiles, masks, values);
//   2. unpack -> pack round trips, in place, with a changed background;
//   3. status codes map to the reference's exception types;
//   4. the tracker constructor rejects what the reference rejects;
//   5. an aligned DiscreteField becomes a dense box holding field(ijk);
//      a non-aligned one is refused;
//   6. advect() either runs on a GPU or fails with an OpenVDB exception;
//   7-8. morphing and filters likewise;
//   9. VolumeAdvection: getMaxVelocity and defaults equal the reference's,
//      the velocity grid's dense box holds getValue at every box voxel;
//  10. volume advect runs on a GPU and equals the reference's result, or
//      fails with an OpenVDB exception.
// Prints "ok <n>" per check; exits non-zero on the first failure.
#include <openvdb/openvdb.h>
#include <openvdb/tools/LevelSetSphere.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "openvdb_gb300/LevelSetAdvect.h"
#include "openvdb_gb300/LevelSetFilter.h"
#include "openvdb_gb300/LevelSetMorph.h"
#include "openvdb_gb300/VolumeAdvect.h"

#include <cmath>

using namespace openvdb;

static int g_n = 0;
#define CHECK(c)                                                              \
    do {                                                                      \
        if (!(c)) {                                                           \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            std::exit(1);                                                     \
        }                                                                     \
    } while (0)

template <class T>
static bool same(const T* a, const T* b, int64_t n) {
    return n == 0 || std::memcmp(a, b, size_t(n) * sizeof(T)) == 0;
}

static bool sameDesc(const gbls_grid_desc& a, const gbls_grid_desc& b) {
    return a.voxel_size == b.voxel_size && a.background == b.background && a.leaf_count == b.leaf_count &&
           a.lower_count == b.lower_count && a.upper_count == b.upper_count &&
           a.root_tile_count == b.root_tile_count && same(a.leaf_origins, b.leaf_origins, 3 * a.leaf_count) &&
           same(a.leaf_masks, b.leaf_masks, 8 * a.leaf_count) &&
           same(a.leaf_values, b.leaf_values, 512 * a.leaf_count) &&
           same(a.lower_origins, b.lower_origins, 3 * a.lower_count) &&
           same(a.lower_tiles, b.lower_tiles, 4096 * a.lower_count) &&
           same(a.upper_origins, b.upper_origins, 3 * a.upper_count) &&
           same(a.upper_tiles, b.upper_tiles, 32768 * a.upper_count) &&
           same(a.root_tile_origins, b.root_tile_origins, 3 * a.root_tile_count) &&
           same(a.root_tile_values, b.root_tile_values, a.root_tile_count);
}

template <class E>
static bool throwsAs(int rc) {
    try {
        openvdb_gb300::detail::check(rc);
    } catch (const E&) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}

int main() {
    namespace og = openvdb_gb300;
    // 1. pack == fixture
    const float center[3] = {3.5f, -7.25f, 1.0f};
    FloatGrid::Ptr sphere = tools::createLevelSetSphere<FloatGrid>(30.0f, Vec3f(center[0], center[1], center[2]), 1.0f, 3.0f);
    og::detail::HostGrid packed = og::detail::pack(*sphere);
    gbls_grid_desc pd = packed.desc();
    gbls_host_grid* fix = nullptr;
    CHECK(gbls_host_sphere(30.0f, center, 1.0f, 3.0f, &fix) == GBLS_OK);
    gbls_grid_desc fd{};
    CHECK(gbls_host_grid_view(fix, &fd) == GBLS_OK);
    CHECK(pd.leaf_count > 100 && pd.upper_count >= 2);
    CHECK(sameDesc(pd, fd));
    std::printf("ok %d pack equals fixture (%lld leaves)\n", ++g_n, (long long)pd.leaf_count);

    // 2. unpack -> pack, into a new grid and in place with another background
    FloatGrid::Ptr copy = FloatGrid::create(0.0f);
    copy->setTransform(sphere->transform().copy());
    og::detail::unpack(packed, *copy);
    og::detail::HostGrid again = og::detail::pack(*copy);
    gbls_grid_desc ad = again.desc();
    CHECK(sameDesc(pd, ad));
    CHECK(copy->activeVoxelCount() == sphere->activeVoxelCount());
    og::detail::HostGrid shifted = packed;
    shifted.background = 4.0f;
    for (float& v : shifted.lower_tiles) v = v > 0.0f ? 4.0f : v < 0.0f ? -4.0f : 0.0f;
    for (float& v : shifted.upper_tiles) v = v > 0.0f ? 4.0f : v < 0.0f ? -4.0f : 0.0f;
    for (float& v : shifted.root_tile_values) v = v > 0.0f ? 4.0f : -4.0f;
    FloatTree* before = &copy->tree();
    og::detail::unpack(shifted, *copy);
    CHECK(&copy->tree() == before && copy->background() == 4.0f);
    og::detail::HostGrid s2 = og::detail::pack(*copy);
    gbls_grid_desc sd = shifted.desc(), s2d = s2.desc();
    CHECK(sameDesc(sd, s2d));
    std::printf("ok %d unpack/pack round trip (in place, background %g)\n", ++g_n, copy->background());

    // 3. status -> exception
    CHECK(throwsAs<ValueError>(GBLS_ERR_VALUE));
    CHECK(throwsAs<RuntimeError>(GBLS_ERR_RUNTIME));
    CHECK(throwsAs<ValueError>(GBLS_ERR_INVALID_ARGUMENT));
    CHECK(throwsAs<NotImplementedError>(GBLS_ERR_UNSUPPORTED));
    CHECK(throwsAs<IndexError>(GBLS_ERR_DOMAIN));
    CHECK(throwsAs<std::bad_alloc>(GBLS_ERR_OUT_OF_MEMORY));
    CHECK(throwsAs<RuntimeError>(GBLS_ERR_CUDA));
    og::detail::check(GBLS_OK);
    og::detail::check(GBLS_ERR_INTERRUPTED);
    std::printf("ok %d status codes map to OpenVDB exceptions\n", ++g_n);

    // 4. tracker constructor checks
    FloatGrid::Ptr fog = FloatGrid::create(0.0f);
    fog->setGridClass(GRID_FOG_VOLUME);
    bool threw = false;
    try {
        og::tools::LevelSetTracker<FloatGrid> t(*fog);
    } catch (const RuntimeError&) {
        threw = true;
    }
    CHECK(threw);
    og::tools::LevelSetTracker<FloatGrid> tracker(*sphere);
    CHECK(tracker.getNormCount() == 3 && tracker.getTemporalScheme() == math::TVD_RK1 &&
          tracker.getHalfWidth() == 3.0f && tracker.leafs().leafCount() == size_t(pd.leaf_count));
    std::printf("ok %d tracker constructor and defaults\n", ++g_n);

    // 5. DiscreteField -> dense box
    Vec3SGrid::Ptr vel = Vec3SGrid::create(Vec3s(0.25f, -0.5f, 1.0f));
    vel->setTransform(sphere->transform().copy());
    vel->tree().setValue(Coord(1, 2, 3), Vec3s(2.0f, 3.0f, 4.0f));
    tools::DiscreteField<Vec3SGrid> field(*vel);
    og::FieldStore fstore;
    std::vector<float>& store = fstore.values;
    gbls_field_desc d = og::FieldTraits<tools::DiscreteField<Vec3SGrid>>::describe(field, *sphere, 0.0f, 1.0f, fstore);
    CHECK(d.kind == GBLS_FIELD_DENSE && d.dense_values == store.data());
    auto at = [&](int x, int y, int z, int c) {
        const size_t i = ((size_t(x - d.dense_origin[0]) * d.dense_dims[1] + size_t(y - d.dense_origin[1])) *
                              d.dense_dims[2] + size_t(z - d.dense_origin[2])) * 3 + c;
        return store[i];
    };
    CHECK(at(1, 2, 3, 0) == 2.0f && at(1, 2, 3, 2) == 4.0f && at(0, 0, 0, 1) == -0.5f);
    CoordBBox band;
    CHECK(sphere->tree().evalActiveVoxelBoundingBox(band));
    for (int a = 0; a < 3; ++a)
        CHECK(d.dense_origin[a] <= band.min()[a] - 8 && d.dense_origin[a] + d.dense_dims[a] - 1 >= band.max()[a] + 8);
    Vec3SGrid::Ptr vel2 = vel->deepCopy();
    vel2->setTransform(math::Transform::createLinearTransform(0.5));
    tools::DiscreteField<Vec3SGrid> field2(*vel2);
    // non-aligned: the grid's own values and transform
    gbls_field_desc d2 = og::FieldTraits<tools::DiscreteField<Vec3SGrid>>::describe(field2, *sphere, 0.0f, 1.0f, fstore);
    CHECK(d2.kind == GBLS_FIELD_DENSE && d2.dense_map_type == 1 + GBLS_MAP_UNIFORM_SCALE && d2.dense_voxel_size == 0.5);
    auto at2 = [&](int x, int y, int z, int c) {
        const size_t i = ((size_t(x - d2.dense_origin[0]) * d2.dense_dims[1] + size_t(y - d2.dense_origin[1])) *
                              d2.dense_dims[2] + size_t(z - d2.dense_origin[2])) * 3 + c;
        return store[i];
    };
    CHECK(at2(1, 2, 3, 1) == 3.0f && at2(0, 0, 0, 2) == 1.0f);
    for (int a = 0; a < 3; ++a)  // the band (world = index at voxel size 1) in 0.5-voxel index space
        CHECK(d2.dense_origin[a] <= 2 * band.min()[a] && d2.dense_origin[a] + d2.dense_dims[a] - 1 >= 2 * band.max()[a]);
    std::printf("ok %d DiscreteField dense box (%d x %d x %d)\n", ++g_n, d.dense_dims[0], d.dense_dims[1], d.dense_dims[2]);

    // 5b. any other functor (the reference's default EnrightField): sampled on
    //     the host at the voxels' world positions, as sample<false> does
    {
        FloatGrid::Ptr unit = tools::createLevelSetSphere<FloatGrid>(0.15f, Vec3f(0.35f), 0.01f, 3.0f);
        tools::EnrightField<float> enright;
        og::FieldStore es;
        const gbls_field_desc de = og::FieldTraits<tools::EnrightField<float>>::describe(enright, *unit, 0.0f, 1.0f, es);
        CHECK(de.kind == GBLS_FIELD_HOST_SAMPLED && de.host_sample && de.host_user == es.context.get());
        const int32_t ijk[6] = {35, 20, 40, -3, 7, 11};
        float v[6];
        de.host_sample(de.host_user, 2, ijk, 0.25f, v);
        bool same = true;
        for (int i = 0; i < 2; ++i) {
            const Vec3f r = enright(unit->transform().indexToWorld(Coord(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2])), 0.25f);
            same = same && v[3 * i] == r[0] && v[3 * i + 1] == r[1] && v[3 * i + 2] == r[2];
        }
        CHECK(same);
        std::printf("ok %d EnrightField sampled on the host like sample<false>\n", ++g_n);
    }

    // 6. advect: runs on a GPU, else an OpenVDB exception (no GPU here)
    og::tools::LevelSetAdvection<FloatGrid, og::ConstantField> adv(*sphere, og::ConstantField{Vec3f(1.0f, 0.5f, 0.25f)});
    adv.setTemporalScheme(math::TVD_RK3);
    adv.setNormCount(1);
    try {
        const size_t n = adv.advect(0.0f, 1.0f);
        std::printf("ok %d advect ran on a device: %zu substeps, %llu active voxels\n", ++g_n, n,
                    (unsigned long long)sphere->activeVoxelCount());
    } catch (const openvdb::Exception& e) {
        std::printf("ok %d advect without a device: %s\n", ++g_n, e.what());
    }
    // 7. morphing: same defaults and range checks as the reference; runs on a
    //    GPU, else an OpenVDB exception
    FloatGrid::Ptr src2 = tools::createLevelSetSphere<FloatGrid>(12.0f, Vec3f(0.0f), 1.0f, 3.0f);
    FloatGrid::Ptr tgt2 = tools::createLevelSetSphere<FloatGrid>(15.0f, Vec3f(2.0f, 1.0f, -1.0f), 1.0f, 3.0f);
    og::tools::LevelSetMorphing<FloatGrid> morph(*src2, *tgt2);
    FloatGrid::Ptr src2ref = src2->deepCopy();
    tools::LevelSetMorphing<FloatGrid> refMorph(*src2ref, *tgt2);
    CHECK(morph.getTemporalScheme() == refMorph.getTemporalScheme() && morph.getNormCount() == refMorph.getNormCount() &&
          morph.minMask() == refMorph.minMask() && morph.maxMask() == refMorph.maxMask());
    threw = false;
    try {
        morph.setMaskRange(1.0f, 1.0f);
    } catch (const ValueError&) {
        threw = true;
    }
    CHECK(threw);
    morph.setMaskRange(-2.0f, 2.0f);
    refMorph.setMaskRange(-2.0f, 2.0f);
    CHECK(morph.minMask() == refMorph.minMask() && morph.maxMask() == refMorph.maxMask());
    try {
        const size_t n = morph.advect(0.0f, 1.0f);
        std::printf("ok %d morph ran on a device: %zu substeps\n", ++g_n, n);
    } catch (const openvdb::Exception& e) {
        std::printf("ok %d morph without a device: %s\n", ++g_n, e.what());
    }
    // 8. filters: the tracker base, mask range checks; a mask that is not a
    //    level set (zero background) is refused with an OpenVDB exception
    og::tools::LevelSetFilter<FloatGrid> filt(*src2);
    CHECK(filt.getNormCount() == 3 && filt.minMask() == 0.0f && filt.maxMask() == 1.0f);
    threw = false;
    try {
        filt.setMaskRange(1.0f, 1.0f);
    } catch (const ValueError&) {
        threw = true;
    }
    CHECK(threw);
    FloatGrid maskGrid(0.0f);
    threw = false;
    try {
        filt.gaussian(1, &maskGrid);
    } catch (const openvdb::Exception&) {
        threw = true;
    }
    CHECK(threw);
    try {
        filt.laplacian();
        std::printf("ok %d filter ran on a device\n", ++g_n);
    } catch (const openvdb::Exception& e) {
        std::printf("ok %d filter without a device: %s\n", ++g_n, e.what());
    }
    // 9. VolumeAdvection
    {
        Vec3fGrid::Ptr vel = Vec3fGrid::create(Vec3f(0.1f, 0.0f, -0.05f));
        auto vacc = vel->getAccessor();
        for (int i = -8; i < 8; ++i)
            for (int j = -8; j < 8; ++j)
                for (int k = -8; k < 8; ++k)
                    vacc.setValue(Coord(i, j, k), Vec3f(0.3f * std::sin(0.2f * float(i)),
                                                        0.2f * std::cos(0.3f * float(j)), 0.1f * float(k) / 8.0f));
        FloatGrid::Ptr fog = FloatGrid::create(0.0f);
        auto facc = fog->getAccessor();
        for (int i = -5; i <= 5; ++i)
            for (int j = -5; j <= 5; ++j)
                for (int k = -5; k <= 5; ++k) {
                    const float r = std::sqrt(float(i * i + j * j + k * k));
                    if (r <= 5.0f) facc.setValue(Coord(i, j, k), 1.0f - r / 5.0f);
                }
        og::tools::VolumeAdvection<Vec3fGrid> va(*vel);
        tools::VolumeAdvection<Vec3fGrid> vr(*vel);
        CHECK(va.getMaxVelocity() == vr.getMaxVelocity() && va.getIntegrator() == vr.getIntegrator() &&
              va.getLimiter() == vr.getLimiter() && va.getSubSteps() == vr.getSubSteps() &&
              va.getMaxDistance(*fog, 1.0) == vr.getMaxDistance(*fog, 1.0));
        std::vector<float> store;
        const gbls_field_desc fd = og::detail::describeVelocityGrid(*vel, *fog, store);
        CHECK(fd.kind == GBLS_FIELD_DENSE && fd.dense_dims[0] == 16 && fd.dense_dims[1] == 16 && fd.dense_dims[2] == 16);
        size_t q = 0;
        bool same_box = true;
        for (int i = -8; i < 8; ++i)
            for (int j = -8; j < 8; ++j)
                for (int k = -8; k < 8; ++k, q += 3) {
                    const Vec3f v = vacc.getValue(Coord(i, j, k));
                    same_box &= store[q] == v[0] && store[q + 1] == v[1] && store[q + 2] == v[2];
                }
        CHECK(same_box && fd.dense_background[0] == 0.1f && fd.dense_map_type == 0);
        std::printf("ok %d VolumeAdvection defaults, max velocity and velocity box\n", ++g_n);
        va.setIntegrator(tools::Scheme::MAC);
        vr.setIntegrator(tools::Scheme::MAC);
        try {
            FloatGrid::Ptr out = va.advect<FloatGrid, tools::Sampler<1, false>>(*fog, 1.0);
            FloatGrid::Ptr ref = vr.advect<FloatGrid, tools::Sampler<1, false>>(*fog, 1.0);
            og::detail::HostGrid a1 = og::detail::pack(*out), b1 = og::detail::pack(*ref);
            CHECK(sameDesc(a1.desc(), b1.desc()));
            std::printf("ok %d volume advect ran on a device, equal to the reference\n", ++g_n);
        } catch (const openvdb::Exception& e) {
            std::printf("ok %d volume advect without a device: %s\n", ++g_n, e.what());
        }
    }
    gbls_host_grid_free(fix);
    return 0;
}
