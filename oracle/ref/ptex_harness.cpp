// ORACLE harness (test infrastructure only): drives the vendored Ptex 2.2 sources (compiled from the
// reference checkout by build_ref.py) to produce golden filter values.
//
// ref_ptex_write  : writes a triangle-mesh, half-float, 3-channel Ptex file with the given per-face data
//                   and adjacency (PtexWriter::open / writeFace / close, Middleware/ptex/Include/Ptexture.h).
// ref_ptex_write_quad : the same for a quad mesh (the separable filter's path, PtexSeparableFilter.cpp).
// ref_ptex_eval   : opens it through a PtexCache and evaluates PtexFilter::getFilter(f_bspline) exactly as
//                   Selas does (Source/Core/Shading/SurfaceParameters.cpp:196-206): eval(result, 0, 3,
//                   faceid, u, v, 0, 0, 0, 0).

#include <cstdint>
#include <cstring>
#include <vector>

#include "PtexHalf.h"
#include "Ptexture.h"

using namespace Ptex;

extern "C" {

// faces: n x 8 ints (log2, texel offset, adj0..2, adjedge0..2); texels: half RGB. Returns 0 on success.
int ref_ptex_write(const char* path, const int32_t* faces, int nfaces, const uint16_t* texels) {
    String err;
    PtexWriter* w = PtexWriter::open(path, mt_triangle, dt_half, 3, -1, nfaces, err, true);
    if (!w) return 1;
    for (int f = 0; f < nfaces; ++f) {
        const int32_t* r = faces + 8 * f;
        const int8_t lg = static_cast<int8_t>(r[0]);
        FaceInfo fi{Res{lg, lg}};
        fi.setadjfaces(r[2], r[3], r[4], -1);
        fi.setadjedges(r[5], r[6], r[7], 0);
        if (!w->writeFace(f, fi, texels + size_t(r[1]) * 3)) {
            w->release();
            return 2;
        }
    }
    bool ok = w->close(err);
    w->release();
    return ok ? 0 : 3;
}

// A quad-mesh texture: faces n x 10 ints (log2, texel offset, adj0..3, adjedge0..3), square faces of 2^log2
// texels a side, half RGB rows of u (PtexWriter with mt_quad).  Returns 0 on success.
int ref_ptex_write_quad(const char* path, const int32_t* faces, int nfaces, const uint16_t* texels) {
    String err;
    PtexWriter* w = PtexWriter::open(path, mt_quad, dt_half, 3, -1, nfaces, err, true);
    if (!w) return 1;
    for (int f = 0; f < nfaces; ++f) {
        const int32_t* r = faces + 10 * f;
        const int8_t lg = static_cast<int8_t>(r[0]);
        FaceInfo fi{Res{lg, lg}};
        fi.setadjfaces(r[2], r[3], r[4], r[5]);
        fi.setadjedges(r[6], r[7], r[8], r[9]);
        if (!w->writeFace(f, fi, texels + size_t(r[1]) * 3)) {
            w->release();
            return 2;
        }
    }
    bool ok = w->close(err);
    w->release();
    return ok ? 0 : 3;
}

// queries: n x (face as int bits, u, v); out: n x 3 (either mesh type: getFilter picks the triangle filter or
// the separable bicubic filter with B-spline weights)
int ref_ptex_eval(const char* path, const float* queries, int n, float* out) {
    String err;
    PtexCache* cache = PtexCache::create(4, 1 << 26, true, nullptr, nullptr);
    PtexTexture* tex = cache->get(path, err);
    if (!tex) {
        cache->release();
        return 1;
    }
    PtexFilter::Options opts(PtexFilter::f_bspline);
    PtexFilter* filter = PtexFilter::getFilter(tex, opts);
    for (int i = 0; i < n; ++i) {
        int32_t face;
        std::memcpy(&face, &queries[3 * i], 4);
        float r[3] = {0, 0, 0};
        filter->eval(r, 0, 3, face, queries[3 * i + 1], queries[3 * i + 2], 0, 0, 0, 0);
        out[3 * i] = r[0];
        out[3 * i + 1] = r[1];
        out[3 * i + 2] = r[2];
    }
    filter->release();
    tex->release();
    cache->release();
    return 0;
}

}  // extern "C"
