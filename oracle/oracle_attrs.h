// ORACLE - test infrastructure only.  Vertex attributes (shading normals, tangents) of the oracle renders' soup,
// set by oracle_set_attributes (oracle_pt.cpp).
#pragma once

#include <cstdint>

namespace ora {

// Indexes the soup of the render about to run (tri_scene may be null: scene 0); returns whether attributes are set.
bool index(const uint32_t* prim, const uint32_t* geom, const uint32_t* tri_scene, int64_t ntri);

// Shading frame of a hit (CalculateSurfaceParams, SurfaceParameters.cpp:157-184) for a mesh of the rendered scene
// itself: the interpolated vertex normal (else ng) normalised, the interpolated tangent with b = cross(n, t) x sign
// (else an orthonormal basis around n).
void frame(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, const float ng[3], float n[3], float t[3],
           float b[3]);

// Base colour of the 2D image bound to mesh (scene, geom) at a hit (the reference's non-Ptex texture path,
// SurfaceParameters.cpp:186-213 with TextureFiltering::Triangle at level 0, Repeat wrapping, sRGB to linear): uvs
// from attribute slot 2 ((0, 0) without them).  False when no image is bound.
bool tex2d(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, float rgb[3]);

}  // namespace ora
