"""Save / load SceneData in .npz fixtures (test helper)."""
from __future__ import annotations

import numpy as np

from illume_gb300.scenedata import Material, Mesh, SceneData, Texture


def scene_to_arrays(s: SceneData, prefix: str = "scene.") -> dict:
    out = {}
    p = prefix
    out[p + "num_meshes"] = np.int32(len(s.meshes))
    for i, m in enumerate(s.meshes):
        out[f"{p}mesh{i}.positions"] = m.positions
        out[f"{p}mesh{i}.tris"] = m.tris
        out[f"{p}mesh{i}.leaf_size"] = np.int32(m.leaf_size)
        if m.normals is not None:
            out[f"{p}mesh{i}.normals"] = m.normals
        if m.texcoords is not None:
            out[f"{p}mesh{i}.texcoords"] = m.texcoords
    out[p + "inst_mesh"] = np.array([x[0] for x in s.instances], np.int32)
    out[p + "inst_material"] = np.array([x[1] for x in s.instances], np.int32)
    out[p + "inst_mats"] = np.array([np.stack(x[2:5]) for x in s.instances], np.float32).reshape(-1, 3, 3, 4)
    out[p + "spheres"] = np.array([list(x[0]) + [x[1], x[2]] for x in s.spheres], np.float32).reshape(-1, 5)
    out[p + "materials"] = np.array([[m.type, m.albedo_tex, m.roughness_tex, m.ior, m.diffuse_fresnel, *m.eta, *m.k,
                                      m.medium, m.distribution] for m in s.materials], np.float64).reshape(-1, 13)
    out[p + "mediums"] = np.array([list(m[0]) + [m[1], m[2], m[3]] for m in s.mediums], np.float32).reshape(-1, 6)
    out[p + "num_textures"] = np.int32(len(s.textures))
    for i, t in enumerate(s.textures):
        out[f"{p}tex{i}.info"] = np.array([t.type, *t.color, *t.off, *t.scale, t.hdr], np.float32)
        if t.texels is not None:
            out[f"{p}tex{i}.texels"] = t.texels
    out[p + "env_tex"] = np.int32(s.env_tex)
    out[p + "camera"] = np.concatenate([np.asarray(s.camera_transform, np.float32).reshape(12),
                                        np.array([s.camera_fov, s.camera_dof, s.camera_aperture], np.float32)])
    out[p + "settings"] = np.array([s.width, s.height, s.ray_bias, s.tonemapper], np.float64)
    return out


def scene_from_arrays(z, prefix: str = "scene.") -> SceneData:
    p = prefix
    s = SceneData()
    for i in range(int(z[p + "num_meshes"])):
        s.meshes.append(Mesh(z[f"{p}mesh{i}.positions"], z[f"{p}mesh{i}.tris"],
                             z[f"{p}mesh{i}.normals"] if f"{p}mesh{i}.normals" in z else None,
                             z[f"{p}mesh{i}.texcoords"] if f"{p}mesh{i}.texcoords" in z else None,
                             int(z[f"{p}mesh{i}.leaf_size"])))
    mats = z[p + "inst_mats"]
    for k, (m, mt) in enumerate(zip(z[p + "inst_mesh"], z[p + "inst_material"])):
        s.instances.append((int(m), int(mt), mats[k, 0], mats[k, 1], mats[k, 2]))
    for row in z[p + "spheres"]:
        s.spheres.append((tuple(float(x) for x in row[:3]), float(row[3]), int(row[4])))
    for r in z[p + "materials"]:
        s.materials.append(Material(int(r[0]), int(r[1]), int(r[2]), float(r[3]), float(r[4]),
                                    tuple(float(x) for x in r[5:8]), tuple(float(x) for x in r[8:11]),
                                    int(r[11]), int(r[12])))
    for r in z[p + "mediums"]:
        s.mediums.append((tuple(float(x) for x in r[:3]), float(r[3]), float(r[4]), int(r[5])))
    for i in range(int(z[p + "num_textures"])):
        info = z[f"{p}tex{i}.info"]
        s.textures.append(Texture(int(info[0]), tuple(float(x) for x in info[1:4]), tuple(float(x) for x in info[4:7]),
                                  tuple(float(x) for x in info[7:9]),
                                  z[f"{p}tex{i}.texels"] if f"{p}tex{i}.texels" in z else None, int(info[9])))
    s.env_tex = int(z[p + "env_tex"])
    cam = z[p + "camera"]
    s.camera_transform = cam[:12].reshape(3, 4).copy()
    s.camera_fov, s.camera_dof, s.camera_aperture = float(cam[12]), float(cam[13]), float(cam[14])
    st = z[p + "settings"]
    s.width, s.height, s.ray_bias, s.tonemapper = int(st[0]), int(st[1]), float(np.float32(st[2])), int(st[3])
    return s
