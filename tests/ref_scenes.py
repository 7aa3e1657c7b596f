"""Scenes whose images and shading values are pinned against the reference's own path tracer
(tests/golden/ref_pt_golden.npz, made by tests/golden/make_golden.py through oracle/_ref/libref_pt.so).

One definition serves the fixture generator and the tests that compare the oracle and the GPU with it.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from selas_gb300 import scenes

SEED = 0x5E1A5000


def checker(n=8):
    y, x = np.mgrid[0:n, 0:n]
    a, b = np.array([0.9, 0.8, 0.1]), np.array([0.1, 0.2, 0.9])
    img = np.where(((x + y) % 2 == 0)[..., None], a, b).astype(np.float32)
    img[0, 0] = [1.0, 0.0, 0.0]  # one odd texel marks the orientation
    return img


def textured_cornell():
    """The Cornell box with a checker image on its floor (geomID 0; uvs 0..2.5, so the image repeats and the
    filter wraps) and a grey image on the back wall without uvs (every hit samples uv (0, 0))."""
    c = scenes.cornell_box()
    v0 = c.geometry.meshes[0][1]
    uvs = (v0[:, [0, 2]] / 556.0 * 2.5).astype(np.float32)
    attrs = {0: {"uvs": uvs}}
    return dataclasses.replace(c, attrs=attrs, textures={0: checker(), 2: np.full((4, 4, 1), 0.35, np.float32)})


def ibl_spheres(rotation=0.0):
    """Ptex-textured displaced spheres on a floor lit by the synthetic sky image (light and miss images)."""
    rs = scenes.textured_spheres(count=4, level=3)
    return dataclasses.replace(rs, ibl=scenes.sky_ibl(rotation=rotation), background=(0.0, 0.0, 0.0))


def media_cornell():
    """The Cornell box with a participating medium: the tall box is a rough dielectric solid (specTrans 1,
    ior 1.5) whose interior scatters isotropically (scatterDistance 0.01, transmittanceColor (0.8, 0.5, 0.3):
    extinction CalculateExtinction(color, distance), Disney.cpp:337-343), and the short box is a smooth
    dielectric without a medium."""
    c = scenes.cornell_box()
    mats = dict(c.materials)
    mats[6] = dict(shader=1, lightSetIndex=0, baseColor=(0.9, 0.9, 0.9), transmittanceColor=(0.8, 0.5, 0.3),
                   specTrans=1.0, roughness=0.2, metallic=0.0, ior=1.5, scatterDistance=0.01)
    mats[5] = dict(shader=1, lightSetIndex=0, baseColor=(0.95, 0.95, 0.95), transmittanceColor=(1.0, 1.0, 1.0),
                   specTrans=1.0, roughness=0.05, metallic=0.0, ior=1.5)
    return dataclasses.replace(c, materials=mats)


# name -> (scene, width, height, spp, max_bounces): the images rendered on PCG32 streams with seed SEED
IMAGES = {
    "cornell": (scenes.cornell_box, 64, 64, 16, 8),
    "media": (media_cornell, 48, 48, 16, 16),
    "smooth": (scenes.smooth_spheres, 48, 48, 8, 6),
    "textured": (textured_cornell, 48, 48, 8, 6),
    "ibl": (lambda: ibl_spheres(0.3), 64, 48, 8, 6),
}

# name -> (scene, width, height, samples per axis, max segments): the deferred path tracer's images on PCG32 streams
# (2D base-colour images are left out: the reference's deferred shading looks every valid texture handle up as a
# Ptex file, DeferredPathTracer.cpp:317-330)
DEFERRED = {
    "cornell": (scenes.cornell_box, 48, 48, 3, 16),
    "media": (media_cornell, 48, 48, 3, 16),
    "smooth": (scenes.smooth_spheres, 48, 48, 3, 12),
    "ibl": (lambda: ibl_spheres(0.3), 64, 48, 3, 16),
}
