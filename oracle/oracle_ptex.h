// ORACLE - test infrastructure only.  The oracle Ptex triangle filter for the oracle integrators.
#pragma once

#include <cstdint>

namespace orp {

// rows: n x 8 ints (log2, texel offset, adj0..2, adjedge0..2); texels: half RGB (not copied).
class Texture {
public:
    Texture(const int32_t* rows, int n, const uint16_t* texels);
    ~Texture();
    bool eval(int face, float u, float v, float* out) const;

private:
    void* faces;
    int nfaces;
    const uint16_t* texels;
};

// rows: n x 10 ints (log2, texel offset, adj0..3, adjedge0..3) of a quad-mesh texture; texels: half RGB (copied,
// with the writer's constant-face flags computed from them).
class QuadTexture {
public:
    QuadTexture(const int32_t* rows, int n, const uint16_t* texels, size_t texel_count);
    ~QuadTexture();
    bool eval(int face, float u, float v, float* out) const;

private:
    void* state;
};

}  // namespace orp
