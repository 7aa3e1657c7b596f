/* ORACLE harness (test infrastructure only): the Embree 3.2 entry points that the reference's scene-loading
 * code (Source/Core/SceneLib/{Scene,Subscene,Model}Resource.cpp) references but the harness never reaches.
 * Scenes are assembled by pt_harness.cpp, not cooked and committed, so each stub aborts if called.  C linkage
 * names carry no signature; the queries themselves (rtcIntersect1, rtcOccluded1, rtcInterpolate) are in
 * pt_harness.cpp. */
#include <stdlib.h>

#define STUB(name) \
    void name(void) { abort(); }

STUB(rtcNewScene)
STUB(rtcCommitScene)
STUB(rtcReleaseScene)
STUB(rtcNewGeometry)
STUB(rtcCommitGeometry)
STUB(rtcReleaseGeometry)
STUB(rtcAttachGeometry)
STUB(rtcAttachGeometryByID)
STUB(rtcSetSharedGeometryBuffer)
STUB(rtcSetGeometryVertexAttributeCount)
STUB(rtcSetGeometryUserData)
STUB(rtcSetGeometryUserPrimitiveCount)
STUB(rtcSetGeometryTransform)
STUB(rtcSetGeometryTimeStepCount)
STUB(rtcSetGeometryOccludedFunction)
STUB(rtcSetGeometryIntersectFunction)
STUB(rtcSetGeometryIntersectFilterFunction)
STUB(rtcSetGeometryInstancedScene)
STUB(rtcSetGeometryBoundsFunction)
