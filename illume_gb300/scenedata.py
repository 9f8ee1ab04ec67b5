"""Flat scene description in numpy arrays, convertible to illume_scene_desc.

SceneData holds what the reference's HostScene holds after parsing a JSON scene
(src/scene/scene.h:20-27): meshes, mesh instances with their transforms, spheres,
materials, mediums, textures, the environment texture, the camera and the
render_settings. It is the in-memory input of illume_scene_create and the exchange
format with test checkers (illume_scene_describe fills one from a loaded scene).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _capi as C


def _i32(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32))


def _f32(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float32))


@dataclass
class Mesh:
    positions: np.ndarray                 # (V, 3) float32
    tris: np.ndarray                      # (T, 3) int32
    normals: Optional[np.ndarray] = None  # (V, 3) float32, None = face normals
    texcoords: Optional[np.ndarray] = None  # (V, 2) float32
    leaf_size: int = 4


@dataclass
class Material:
    type: int
    albedo_tex: int
    roughness_tex: int
    ior: float = 0.0
    diffuse_fresnel: float = 0.0
    eta: tuple = (0.0, 0.0, 0.0)
    k: tuple = (0.0, 0.0, 0.0)
    medium: int = -1
    distribution: int = C.DIST_BECKMANN


@dataclass
class Texture:
    type: int
    color: tuple = (0.0, 0.0, 0.0)
    off: tuple = (0.0, 0.0, 0.0)
    scale: tuple = (1.0, 1.0)
    texels: Optional[np.ndarray] = None   # (H, W, 4) float32 RGBA
    hdr: int = 1


def affine_inverse(m34: np.ndarray) -> np.ndarray:
    m = np.eye(4)
    m[:3, :] = m34
    return np.linalg.inv(m)[:3, :].astype(np.float32)


def normal_matrix(inv34: np.ndarray) -> np.ndarray:
    """Transpose of the inverse (the reference's trans_inv), as 3x4 rows."""
    m = np.eye(4)
    m[:3, :] = inv34
    return m.T[:3, :].astype(np.float32)


@dataclass
class SceneData:
    meshes: List[Mesh] = field(default_factory=list)
    instances: list = field(default_factory=list)   # (mesh, material, mat34, inv34, trans_inv34)
    spheres: list = field(default_factory=list)     # (center(3), radius, material)
    materials: List[Material] = field(default_factory=list)
    mediums: list = field(default_factory=list)     # (absorption(3) already 1-json, scattering, g, active)
    textures: List[Texture] = field(default_factory=list)
    env_tex: int = -1
    camera_transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32)[:3].copy())
    camera_fov: float = 40.0
    camera_dof: float = 1.0
    camera_aperture: float = 0.0
    width: int = 512
    height: int = 512
    ray_bias: float = 0.0
    tonemapper: int = C.TONE_LINEAR

    # ---- builders ----
    def add_texture(self, tex: Texture) -> int:
        self.textures.append(tex)
        return len(self.textures) - 1

    def constant(self, rgb) -> int:
        return self.add_texture(Texture(C.TEX_CONSTANT, color=tuple(float(v) for v in rgb)))

    def add_material(self, mat: Material) -> int:
        self.materials.append(mat)
        return len(self.materials) - 1

    def add_mesh(self, mesh: Mesh) -> int:
        self.meshes.append(mesh)
        return len(self.meshes) - 1

    def add_instance(self, mesh: int, material: int, mat34=None) -> int:
        m = np.eye(4, dtype=np.float32)[:3].copy() if mat34 is None else _f32(mat34).reshape(3, 4)
        inv = affine_inverse(m)
        self.instances.append((mesh, material, m, inv, normal_matrix(inv)))
        return len(self.instances) - 1

    def add_sphere(self, center, radius, material) -> int:
        self.spheres.append((tuple(float(c) for c in center), float(radius), int(material)))
        return len(self.spheres) - 1

    def add_medium(self, absorption, scattering, g) -> int:
        a = np.asarray(absorption, dtype=np.float32)
        active = int(float(np.dot(a, a)) > 1e-5 or scattering > 0)
        self.mediums.append((tuple(float(v) for v in a), float(scattering), float(g), active))
        return len(self.mediums) - 1

    def num_triangles(self) -> int:
        return int(sum(len(m.tris) for m in self.meshes))

    # ---- conversion ----
    def to_desc(self):
        """Return (SceneDesc, keepalive) with pointers into arrays owned by keepalive."""
        keep = []

        def arr(a, kind):
            a = _i32(a) if kind == "i" else (np.ascontiguousarray(np.asarray(a, dtype=np.int64)) if kind == "l" else _f32(a))
            keep.append(a)
            ptype = {"i": ctypes.c_int32, "l": ctypes.c_int64, "f": ctypes.c_float}[kind]
            return a.ctypes.data_as(ctypes.POINTER(ptype))

        d = C.SceneDesc()
        nm = len(self.meshes)
        d.num_meshes = nm
        vo, to, nv, nt, pos, nrm, tcs, tri = [], [], [], [], [], [], [], []
        v = t = 0
        for m in self.meshes:
            V, T = len(m.positions), len(m.tris)
            vo.append(v); to.append(t); nv.append(V); nt.append(T)
            pos.append(_f32(m.positions).reshape(-1, 3))
            nrm.append(_f32(m.normals).reshape(-1, 3) if m.normals is not None else np.zeros((V, 3), np.float32))
            tcs.append(_f32(m.texcoords).reshape(-1, 2) if m.texcoords is not None else np.zeros((V, 2), np.float32))
            tri.append(_i32(m.tris).reshape(-1, 3))
            v += V; t += T
        cat = lambda L, shape: np.concatenate(L) if L else np.zeros(shape)
        d.mesh_vertex_offset = arr(vo or [0], "i")
        d.mesh_num_vertices = arr(nv or [0], "i")
        d.mesh_tri_offset = arr(to or [0], "i")
        d.mesh_num_tris = arr(nt or [0], "i")
        d.mesh_has_normals = arr([int(m.normals is not None) for m in self.meshes] or [0], "i")
        d.mesh_has_texcoords = arr([int(m.texcoords is not None) for m in self.meshes] or [0], "i")
        d.mesh_bvh_leaf_size = arr([int(m.leaf_size) for m in self.meshes] or [4], "i")
        d.positions = arr(cat(pos, (1, 3)), "f")
        d.normals = arr(cat(nrm, (1, 3)), "f")
        d.texcoords = arr(cat(tcs, (1, 2)), "f")
        d.tris = arr(cat(tri, (1, 3)), "i")

        d.num_instances = len(self.instances)
        ins = self.instances or [(0, 0, np.zeros((3, 4)), np.zeros((3, 4)), np.zeros((3, 4)))]
        d.inst_mesh = arr([i[0] for i in ins], "i")
        d.inst_material = arr([i[1] for i in ins], "i")
        d.inst_mat = arr(np.stack([i[2] for i in ins]), "f")
        d.inst_inv = arr(np.stack([i[3] for i in ins]), "f")
        d.inst_trans_inv = arr(np.stack([i[4] for i in ins]), "f")

        d.num_spheres = len(self.spheres)
        sp = self.spheres or [((0, 0, 0), 0, 0)]
        d.sphere_center_radius = arr([list(s[0]) + [s[1]] for s in sp], "f")
        d.sphere_material = arr([s[2] for s in sp], "i")

        d.num_materials = len(self.materials)
        ms = self.materials or [Material(C.MAT_LAMBERT, 0, 0)]
        d.mat_type = arr([m.type for m in ms], "i")
        d.mat_albedo_tex = arr([m.albedo_tex for m in ms], "i")
        d.mat_roughness_tex = arr([m.roughness_tex for m in ms], "i")
        d.mat_medium = arr([m.medium for m in ms], "i")
        d.mat_distribution = arr([m.distribution for m in ms], "i")
        d.mat_ior = arr([m.ior for m in ms], "f")
        d.mat_diffuse_fresnel = arr([m.diffuse_fresnel for m in ms], "f")
        d.mat_eta = arr([list(m.eta) for m in ms], "f")
        d.mat_k = arr([list(m.k) for m in ms], "f")

        d.num_mediums = len(self.mediums)
        md = self.mediums or [((0, 0, 0), 0.0, 0.0, 0)]
        d.med_absorption = arr([list(m[0]) for m in md], "f")
        d.med_scattering = arr([m[1] for m in md], "f")
        d.med_g = arr([m[2] for m in md], "f")
        d.med_active = arr([m[3] for m in md], "i")

        d.num_textures = len(self.textures)
        tx = self.textures or [Texture(C.TEX_CONSTANT)]
        offs, pool, o = [], [], 0
        for tt in tx:
            offs.append(o)
            if tt.type == C.TEX_BITMAP:
                flat = _f32(tt.texels).reshape(-1)
                pool.append(flat)
                o += flat.size
        d.tex_type = arr([tt.type for tt in tx], "i")
        d.tex_color = arr([list(tt.color) for tt in tx], "f")
        d.tex_off = arr([list(tt.off) for tt in tx], "f")
        d.tex_scale = arr([list(tt.scale) for tt in tx], "f")
        d.tex_width = arr([tt.texels.shape[1] if tt.type == C.TEX_BITMAP else 0 for tt in tx], "i")
        d.tex_height = arr([tt.texels.shape[0] if tt.type == C.TEX_BITMAP else 0 for tt in tx], "i")
        d.tex_hdr = arr([tt.hdr for tt in tx], "i")
        d.tex_texel_offset = arr(offs, "l")
        d.texels = arr(np.concatenate(pool) if pool else np.zeros(4, np.float32), "f")
        d.env_tex = self.env_tex

        ct = _f32(self.camera_transform).reshape(12)
        for i in range(12):
            d.camera_transform[i] = float(ct[i])
        d.camera_fov = self.camera_fov
        d.camera_dof = self.camera_dof
        d.camera_aperture = self.camera_aperture
        d.width, d.height = self.width, self.height
        d.ray_bias = self.ray_bias
        d.tonemapper = self.tonemapper
        return d, keep

    @staticmethod
    def from_desc(d: "C.SceneDesc") -> "SceneData":
        """Copy a described scene (pointers valid while its owner lives) into numpy arrays."""
        def get(ptr, n, dtype, shape=None):
            if n <= 0 or not ptr:
                return np.zeros((0,) if shape is None else (0,) + shape, dtype)
            a = np.ctypeslib.as_array(ptr, shape=(n * (int(np.prod(shape)) if shape else 1),)).astype(dtype).copy()
            return a.reshape((n,) + shape) if shape else a

        s = SceneData()
        nm = d.num_meshes
        vo = get(d.mesh_vertex_offset, nm, np.int32)
        nv = get(d.mesh_num_vertices, nm, np.int32)
        to = get(d.mesh_tri_offset, nm, np.int32)
        nt = get(d.mesh_num_tris, nm, np.int32)
        hn = get(d.mesh_has_normals, nm, np.int32)
        ht = get(d.mesh_has_texcoords, nm, np.int32)
        ls = get(d.mesh_bvh_leaf_size, nm, np.int32)
        vtot = int((vo + nv).max()) if nm else 0
        ttot = int((to + nt).max()) if nm else 0
        P = get(d.positions, vtot, np.float32, (3,))
        N = get(d.normals, vtot, np.float32, (3,))
        T = get(d.texcoords, vtot, np.float32, (2,))
        TR = get(d.tris, ttot, np.int32, (3,))
        for i in range(nm):
            a, b = vo[i], vo[i] + nv[i]
            s.meshes.append(Mesh(P[a:b].copy(), TR[to[i]:to[i] + nt[i]].copy(),
                                 N[a:b].copy() if hn[i] else None, T[a:b].copy() if ht[i] else None, int(ls[i])))
        ni = d.num_instances
        im = get(d.inst_mesh, ni, np.int32)
        imt = get(d.inst_material, ni, np.int32)
        M = get(d.inst_mat, ni, np.float32, (3, 4))
        IV = get(d.inst_inv, ni, np.float32, (3, 4))
        TI = get(d.inst_trans_inv, ni, np.float32, (3, 4))
        for i in range(ni):
            s.instances.append((int(im[i]), int(imt[i]), M[i], IV[i], TI[i]))
        ns = d.num_spheres
        scr = get(d.sphere_center_radius, ns, np.float32, (4,))
        smat = get(d.sphere_material, ns, np.int32)
        for i in range(ns):
            s.spheres.append((tuple(float(x) for x in scr[i, :3]), float(scr[i, 3]), int(smat[i])))
        nmat = d.num_materials
        cols = [get(getattr(d, f), nmat, np.int32) for f in ("mat_type", "mat_albedo_tex", "mat_roughness_tex",
                                                              "mat_medium", "mat_distribution")]
        ior = get(d.mat_ior, nmat, np.float32)
        dfr = get(d.mat_diffuse_fresnel, nmat, np.float32)
        eta = get(d.mat_eta, nmat, np.float32, (3,))
        kk = get(d.mat_k, nmat, np.float32, (3,))
        for i in range(nmat):
            s.materials.append(Material(int(cols[0][i]), int(cols[1][i]), int(cols[2][i]), float(ior[i]), float(dfr[i]),
                                        tuple(float(x) for x in eta[i]), tuple(float(x) for x in kk[i]),
                                        int(cols[3][i]), int(cols[4][i])))
        nmed = d.num_mediums
        ab = get(d.med_absorption, nmed, np.float32, (3,))
        sc = get(d.med_scattering, nmed, np.float32)
        g = get(d.med_g, nmed, np.float32)
        act = get(d.med_active, nmed, np.int32)
        for i in range(nmed):
            s.mediums.append((tuple(float(x) for x in ab[i]), float(sc[i]), float(g[i]), int(act[i])))
        ntx = d.num_textures
        tt = get(d.tex_type, ntx, np.int32)
        tc = get(d.tex_color, ntx, np.float32, (3,))
        tof = get(d.tex_off, ntx, np.float32, (3,))
        tsc = get(d.tex_scale, ntx, np.float32, (2,))
        tw = get(d.tex_width, ntx, np.int32)
        th = get(d.tex_height, ntx, np.int32)
        thdr = get(d.tex_hdr, ntx, np.int32)
        toff = get(d.tex_texel_offset, ntx, np.int64)
        for i in range(ntx):
            texels = None
            if tt[i] == C.TEX_BITMAP:
                n = int(tw[i]) * int(th[i]) * 4
                base = ctypes.cast(d.texels, ctypes.c_void_p).value + int(toff[i]) * 4
                texels = np.ctypeslib.as_array(ctypes.cast(base, ctypes.POINTER(ctypes.c_float)), shape=(n,)).copy()
                texels = texels.reshape(int(th[i]), int(tw[i]), 4)
            s.textures.append(Texture(int(tt[i]), tuple(float(x) for x in tc[i]), tuple(float(x) for x in tof[i]),
                                      tuple(float(x) for x in tsc[i]), texels, int(thdr[i])))
        s.env_tex = int(d.env_tex)
        s.camera_transform = np.array(list(d.camera_transform), np.float32).reshape(3, 4)
        s.camera_fov, s.camera_dof, s.camera_aperture = float(d.camera_fov), float(d.camera_dof), float(d.camera_aperture)
        s.width, s.height = int(d.width), int(d.height)
        s.ray_bias = float(d.ray_bias)
        s.tonemapper = int(d.tonemapper)
        return s
