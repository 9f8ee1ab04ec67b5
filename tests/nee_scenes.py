"""Scenes of the next-event estimator's tests (GPU and oracle)."""
import numpy as np

from illume_gb300 import _capi as C


def textured_emitter_scene():
    """Rough dielectric reflection and lambert surfaces lit by a checker-textured emissive
    quad and a dim constant environment."""
    from illume_gb300 import synth
    from illume_gb300.scenedata import Material, Mesh, SceneData, Texture
    s = SceneData()
    P, T, UV = synth.quad(4.0, 0.0)
    floor = s.add_mesh(Mesh(P, T, texcoords=UV))
    lam = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.7, 0.6, 0.5)), s.constant((1e-4,) * 3)))
    rr = s.add_material(Material(C.MAT_ROUGHREFLECTIVE, s.constant((1, 1, 1)), s.constant((0.3,) * 3), ior=1.5,
                                 distribution=C.DIST_GGX))
    chk = s.add_texture(Texture(C.TEX_CHECKERBOARD, color=(6.0, 5.0, 4.0), off=(1.0, 1.0, 2.0), scale=(4.0, 4.0)))
    light = s.add_material(Material(C.MAT_EMISSIVE, chk, s.constant((0, 0, 0))))
    s.add_instance(floor, lam)
    M = np.zeros((3, 4))
    M[:, :3] = np.diag([0.4, 1.0, 0.4])
    M[:, 3] = (0.3, 2.0, 0.2)
    s.add_instance(floor, light, M.astype(np.float32))
    Pi, Ti = synth.displaced_icosphere(synth.freq_for_tris(2000), 9, amp=0.1, radius=0.6)
    ball = s.add_mesh(Mesh(Pi, Ti))
    Mb = np.zeros((3, 4))
    Mb[:, :3] = np.eye(3)
    Mb[:, 3] = (0.0, 0.6, 0.0)
    s.add_instance(ball, rr, Mb.astype(np.float32))
    s.env_tex = s.constant((0.05, 0.07, 0.1))
    s.camera_transform = synth.lookat((0.0, 1.6, -3.2), (0.0, 0.5, 0.0))
    s.width = s.height = 24
    s.ray_bias = 1e-4
    return s


def env_scene():
    """The traversal scene (rough gold, checkerboard ground) under a softer sun (peak 50,
    5 degrees) so that the reference estimator's sun hits are not too rare for a 3-sigma
    comparison at test sample counts."""
    from illume_gb300 import synth
    from illume_gb300.scenedata import Texture
    sd = synth.traversal_scene(tris=5000, env_size=(16, 8), width=24, height=24)
    sd.textures[sd.env_tex] = Texture(C.TEX_BITMAP, texels=synth.environment_map(1, 256, 128, sun_peak=50.0,
                                                                                  sun_sigma_deg=5.0), hdr=1)
    return sd


def cornell():
    from illume_gb300 import synth
    return synth.cornell_scene(24, 24)


SCENES = {"cornell": cornell, "environment": env_scene, "textured_emitter": textured_emitter_scene}
