// ORACLE - test infrastructure only.  The image-based light set by oracle_set_ibl (oracle_pt.cpp) seen as the VCM
// oracle's environment emitter.
#pragma once

namespace ora {

bool env_present();

// A direction toward the environment from four uniforms: a texel by the marginal and conditional CDFs of
// sin(theta) x luma (BuildImageBasedLight.cpp:18-107), jittered over the directions that look the texel up.
void env_direction(float r0, float r1, float r2, float r3, float dir[3]);

// Solid-angle density of env_direction at `dir`.
float env_pdf(const float dir[3]);

// The light image times the exposure at `dir` (SampleIbl, ImageBasedLightResource.cpp:154-195).
void env_radiance(const float dir[3], float rad[3]);

// The miss image at `dir` (SampleIblMiss, ImageBasedLightResource.cpp:198-218): what camera rays and pure-specular
// camera chains see.
void env_miss(const float dir[3], float rad[3]);

}  // namespace ora
