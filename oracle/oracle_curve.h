// ORACLE - test infrastructure only.  Round B-spline curve geometries of the render oracle's scenes
// (oracle_set_curves in oracle_curve.cpp), queried beside each scene's triangles.
#pragma once

#include <cstdint>

namespace orcv {

bool any(uint32_t scene);
// World box of the scene's curves (false: none).
bool bounds(uint32_t scene, float lo[3], float hi[3]);
// Nearest curve hit with tnear <= t <= tfar, ties to the smaller (geomID, primID): t, u, Ng, primID, geomID.
bool closest(uint32_t scene, const float* org, const float* dir, float tnear, float tfar, float& t, float& u,
             float ng[3], uint32_t& prim, uint32_t& geom);
bool occluded(uint32_t scene, const float* org, const float* dir, float tnear, float tfar);

}  // namespace orcv
