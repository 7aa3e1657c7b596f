// ORACLE - test infrastructure only.  Vertex attributes (shading normals, tangents) of the oracle renders' soup,
// set by oracle_set_attributes (oracle_pt.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace ora {

// Indexes the soup of the render about to run (tri_scene may be null: scene 0); returns whether attributes are set.
bool index(const uint32_t* prim, const uint32_t* geom, const uint32_t* tri_scene, int64_t ntri);

// Shading frame of a hit (CalculateSurfaceParams, SurfaceParameters.cpp:157-184) for a mesh of the rendered scene
// itself: the interpolated vertex normal (else ng) normalised, the interpolated tangent with b = cross(n, t) x sign
// (else an orthonormal basis around n).
void frame(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, const float ng[3], float n[3], float t[3],
           float b[3]);
// The same for a mesh inside instances: normal and tangent through the entered instances' local-to-world rows
// (l2w0 outer, l2w1 inner; null where none), innermost first.
void frame_through(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, const float ng[3], const float* l2w0,
                   const float* l2w1, float n[3], float t[3], float b[3]);

// Base colour of the 2D image bound to mesh (scene, geom) at a hit (the reference's non-Ptex texture path,
// SurfaceParameters.cpp:186-213 with TextureFiltering::Triangle at level 0, Repeat wrapping, sRGB to linear): uvs
// from attribute slot 2 ((0, 0) without them).  False when no image is bound.
bool tex2d(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, float rgb[3]);
// the quad-mesh Ptex bound to (scene, geom) at soup triangle prim (2 * quad + half) with its barycentrics; false
// when none is bound
bool quad_ptex(uint32_t scene, uint32_t geom, uint32_t prim, float u, float v, float rgb[3]);

// One component k of a vertex attribute at a hit, from the soup's corner arrays (`per` floats per corner, three
// corners per soup triangle): (1 - u - v) a0 + u a1 + v a2 on a triangle; on a quad mesh (flags bit 8, soup
// triangles 2q = (v0, v1, v3) and 2q + 1 = (v2, v3, v1)) bilinearly, t_uv = (1 - v)((1 - u) t0 + u t1) +
// v((1 - u) t3 + u t2), at the quad's (u, v) (RTC_GEOMETRY_TYPE_QUAD.3embree3: the second triangle's
// (u', v') -> (1 - u', 1 - v')).
float corner_interp(const std::vector<float>& arr, int per, int64_t tri, uint8_t flags, uint32_t prim, float u, float v,
                    int k);

}  // namespace ora
