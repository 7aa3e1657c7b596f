// Compiled check of the drop-in boundary (include/selas.h against Embree 3.2's C API, which the reference binds:
// Middleware/embree-latest/include/embree3/rtcore_ray.h:26-63, rtcore_common.h:66,72).
//
// Built with -DSEL_CHECK_EMBREE_LAYOUT and the reference's Embree headers on the include path, every field of
// RTCRay, RTCHit and RTCRayHit is asserted at compile time to sit at the offset, with the size, of its SelRay /
// SelHit / SelRayHit counterpart; without that define only selas.h is needed.  Run (with a GPU), it performs the
// calls INTEGRATION.md shows on a two-triangle scene: records laid out by the Embree structs (or the Sel ones)
// go through sel_intersect1 / sel_occluded1 / sel_intersect1M (dense and embedded in a larger caller struct) /
// sel_occluded1M unchanged, and the hits come back where the reference's RayPick reads them
// (Source/Applications/Selas/Source/PathTracer.cpp:118-130).  Exit status 0 and "boundary ok" on success.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <vector>

#include "selas.h"

#ifdef SEL_CHECK_EMBREE_LAYOUT
#include "embree3/rtcore_ray.h"

#define SAME_FIELD(A, B, f) \
    static_assert(offsetof(A, f) == offsetof(B, f) && sizeof(((A*)0)->f) == sizeof(((B*)0)->f), #A "." #f)
static_assert(sizeof(RTCRay) == sizeof(SelRay) && alignof(RTCRay) == alignof(SelRay), "RTCRay size / alignment");
SAME_FIELD(RTCRay, SelRay, org_x);
SAME_FIELD(RTCRay, SelRay, org_y);
SAME_FIELD(RTCRay, SelRay, org_z);
SAME_FIELD(RTCRay, SelRay, tnear);
SAME_FIELD(RTCRay, SelRay, dir_x);
SAME_FIELD(RTCRay, SelRay, dir_y);
SAME_FIELD(RTCRay, SelRay, dir_z);
SAME_FIELD(RTCRay, SelRay, time);
SAME_FIELD(RTCRay, SelRay, tfar);
SAME_FIELD(RTCRay, SelRay, mask);
SAME_FIELD(RTCRay, SelRay, id);
SAME_FIELD(RTCRay, SelRay, flags);
static_assert(sizeof(RTCHit) == sizeof(SelHit), "RTCHit size");
SAME_FIELD(RTCHit, SelHit, Ng_x);
SAME_FIELD(RTCHit, SelHit, Ng_y);
SAME_FIELD(RTCHit, SelHit, Ng_z);
SAME_FIELD(RTCHit, SelHit, u);
SAME_FIELD(RTCHit, SelHit, v);
SAME_FIELD(RTCHit, SelHit, primID);
SAME_FIELD(RTCHit, SelHit, geomID);
SAME_FIELD(RTCHit, SelHit, instID);
static_assert(sizeof(RTCRayHit) == sizeof(SelRayHit) && alignof(RTCRayHit) == alignof(SelRayHit), "RTCRayHit");
SAME_FIELD(RTCRayHit, SelRayHit, ray);
SAME_FIELD(RTCRayHit, SelRayHit, hit);
static_assert(RTC_INVALID_GEOMETRY_ID == SEL_INVALID_GEOMETRY_ID, "invalid id");
static_assert(RTC_MAX_INSTANCE_LEVEL_COUNT == SEL_MAX_INSTANCE_LEVEL_COUNT, "instance levels");
typedef RTCRay CallerRay;
typedef RTCRayHit CallerRayHit;
#else
typedef SelRay CallerRay;
typedef SelRayHit CallerRayHit;
#endif

namespace {

int failures = 0;

void expect(bool ok, const char* what) {
    if (!ok) {
        std::printf("FAILED: %s (%s)\n", what, sel_get_last_error());
        ++failures;
    }
}

// RayPick's record set-up (PathTracer.cpp:101-114).
void make_rayhit(CallerRayHit& r, float ox, float oy, float oz, float dx, float dy, float dz) {
    std::memset(&r, 0, sizeof(r));
    r.ray.org_x = ox; r.ray.org_y = oy; r.ray.org_z = oz;
    r.ray.dir_x = dx; r.ray.dir_y = dy; r.ray.dir_z = dz;
    r.ray.tnear = 0.0f;
    r.ray.tfar = INFINITY;
    r.hit.geomID = SEL_INVALID_GEOMETRY_ID;
    r.hit.primID = SEL_INVALID_GEOMETRY_ID;
    r.hit.instID[0] = SEL_INVALID_GEOMETRY_ID;
    r.hit.instID[1] = SEL_INVALID_GEOMETRY_ID;
}

}  // namespace

int main() {
    SelDevice dev = nullptr;
    if (sel_device_new(0, &dev) != SEL_OK) {
        std::printf("no device: %s\n", sel_get_last_error());
        return 2;
    }
    SelScene scene = nullptr;
    expect(sel_scene_new(dev, &scene) == SEL_OK, "sel_scene_new");
    // a unit square in the z = 5 plane as geomID 7 (two triangles)
    const float verts[4][3] = {{-1, -1, 5}, {1, -1, 5}, {1, 1, 5}, {-1, 1, 5}};
    const unsigned idx[2][3] = {{0, 1, 2}, {0, 2, 3}};
    expect(sel_scene_attach_triangle_mesh(scene, 7, &verts[0][0], 4, sizeof(verts[0]), &idx[0][0], 2) == SEL_OK,
           "attach");
    expect(sel_scene_commit(scene) == SEL_OK, "commit");

    // rtcIntersect1 -> sel_intersect1 on the caller's own record
    CallerRayHit rh;
    make_rayhit(rh, 0.25f, -0.5f, 0.0f, 0.0f, 0.0f, 1.0f);
    expect(sel_intersect1(scene, reinterpret_cast<SelRayHit*>(&rh)) == SEL_OK, "sel_intersect1");
    expect(rh.hit.geomID == 7u && rh.ray.tfar == 5.0f && rh.hit.Ng_z != 0.0f, "closest hit fields");
    const float px = rh.ray.org_x + rh.ray.tfar * rh.ray.dir_x;  // RayPick's hit position
    expect(std::fabs(px - 0.25f) < 1e-6f, "hit position");
    expect(rh.hit.instID[0] == SEL_INVALID_GEOMETRY_ID, "instID of a flat scene");
    CallerRayHit miss;
    make_rayhit(miss, 3.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f);
    expect(sel_intersect1(scene, reinterpret_cast<SelRayHit*>(&miss)) == SEL_OK, "sel_intersect1 (miss)");
    expect(miss.hit.geomID == SEL_INVALID_GEOMETRY_ID && std::isinf(miss.ray.tfar), "a miss leaves the record");

    // rtcOccluded1 -> sel_occluded1: hit <=> tfar = -inf (OcclusionRay, PathTracer.cpp:70-92)
    CallerRay ray;
    std::memset(&ray, 0, sizeof(ray));
    ray.org_x = 0.0f; ray.org_y = 0.0f; ray.org_z = 0.0f; ray.dir_z = 1.0f; ray.tnear = 0.0f; ray.tfar = 10.0f;
    expect(sel_occluded1(scene, reinterpret_cast<SelRay*>(&ray)) == SEL_OK, "sel_occluded1");
    expect(ray.tfar == -INFINITY, "occluded");
    ray.tfar = 4.0f;
    expect(sel_occluded1(scene, reinterpret_cast<SelRay*>(&ray)) == SEL_OK, "sel_occluded1 (short)");
    expect(ray.tfar == 4.0f, "not occluded before the square");

    // batches: dense, and embedded in a caller struct (any stride >= the record size)
    struct Embedded {
        CallerRayHit rh;
        int payload[8];
    };
    const unsigned n = 1000;
    std::vector<Embedded> batch(n);
    std::vector<CallerRayHit> dense(n);
    for (unsigned i = 0; i < n; ++i) {
        const float x = -1.5f + 3.0f * float(i) / float(n);
        make_rayhit(batch[i].rh, x, 0.1f, 0.0f, 0.0f, 0.0f, 1.0f);
        make_rayhit(dense[i], x, 0.1f, 0.0f, 0.0f, 0.0f, 1.0f);
        batch[i].payload[0] = int(i);
    }
    expect(sel_intersect1M(scene, reinterpret_cast<SelRayHit*>(&batch[0].rh), n, sizeof(Embedded)) == SEL_OK,
           "sel_intersect1M (embedded)");
    expect(sel_intersect1M(scene, reinterpret_cast<SelRayHit*>(dense.data()), n, sizeof(CallerRayHit)) == SEL_OK,
           "sel_intersect1M (dense)");
    unsigned hits = 0;
    for (unsigned i = 0; i < n; ++i) {
        const bool inside = std::fabs(dense[i].ray.org_x) <= 1.0f;
        hits += dense[i].hit.geomID == 7u;
        expect(std::memcmp(&dense[i], &batch[i].rh, sizeof(CallerRayHit)) == 0, "embedded and dense agree");
        expect(batch[i].payload[0] == int(i), "the caller's payload is untouched");
        if (inside != (dense[i].hit.geomID == 7u) && std::fabs(std::fabs(dense[i].ray.org_x) - 1.0f) > 1e-5f)
            expect(false, "hit pattern");
    }
    expect(hits > 600 && hits < 700, "hits in the batch");
    std::vector<CallerRay> rays(n);
    for (unsigned i = 0; i < n; ++i) {
        rays[i] = dense[i].ray;
        rays[i].tfar = 100.0f;
    }
    expect(sel_occluded1M(scene, reinterpret_cast<SelRay*>(rays.data()), n, sizeof(CallerRay)) == SEL_OK,
           "sel_occluded1M");
    for (unsigned i = 0; i < n; ++i)
        expect((rays[i].tfar == -INFINITY) == (dense[i].hit.geomID == 7u), "any hit agrees with closest hit");

    expect(sel_scene_release(scene) == SEL_OK, "release scene");
    expect(sel_device_release(dev) == SEL_OK, "release device");
    if (failures) {
        std::printf("%d failures\n", failures);
        return 1;
    }
    std::printf("boundary ok\n");
    return 0;
}
