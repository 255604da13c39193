"""The renderer's camera uniform for cf_render_lit, filled as the reference's
Renderer::uniform does (src/render/mod.rs:162-180) from an orbit camera
(Camera::eye / view_proj, :35-47: a right-handed look-at toward the target
with z up, and a perspective projection with depth in [0, 1], near 0.01,
far 20)."""
import numpy as np

from . import capi


def look_at_rh(eye, target, up):
    f = target - eye
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.identity(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective_rh_zo(fov, aspect, near, far):
    hh = 1.0 / np.tan(0.5 * fov)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = hh / aspect, hh
    m[2, 2], m[2, 3] = far / (near - far), near * far / (near - far)
    m[3, 2] = -1.0
    return m


def render_cam(film_w, film_h, width_m, height_m, top, yaw=0.6, pitch=0.85, dist=None, fov=0.8, aspect=16 / 9,
               target=None, light=(0.45, -0.3, 0.84), intensity=3.0, sky=(0.55, 0.62, 0.7),
               ground=(0.2, 0.18, 0.16), contact_angle_deg=35.0, ortho=False, beauty=False, footprint=0.0,
               lens=None):
    """A cf_render_cam for a film of film_w x film_h cells covering width_m x
    height_m metres, whose relief tops out at `top` (max(h_max, s_max) +
    0.5 mm).  `lens` = (aperture x, aperture y, focus distance) turns on the
    thin lens."""
    dx = np.float32(width_m) / np.float32(film_w)
    tgt = np.array([0.5 * width_m, 0.5 * height_m, 0.0]) if target is None else np.asarray(target, float)
    d = 1.6 * width_m if dist is None else dist
    eye = tgt + d * np.array([np.cos(pitch) * np.cos(yaw), np.cos(pitch) * np.sin(yaw), np.sin(pitch)])
    vp = perspective_rh_zo(fov, aspect, 0.01, 20.0) @ look_at_rh(eye, tgt, np.array([0.0, 0.0, 1.0]))
    inv = np.linalg.inv(vp)
    c = capi.RenderCam()
    for k, v in enumerate(inv.T.reshape(-1)):
        c.inv_vp[k] = v
    for k, v in enumerate(vp.T.reshape(-1)):
        c.vp[k] = v
    c.eye[:] = [eye[0], eye[1], eye[2], 0.0]
    c.canvas[:] = [width_m, height_m, dx, top]
    ln = np.asarray(light, float)
    ln = ln / np.linalg.norm(ln)
    c.light[:] = [ln[0], ln[1], ln[2], intensity]
    c.size[:] = [film_w, film_h, 0, 0]
    c.sky[:] = [sky[0], sky[1], sky[2], 1.0]
    c.ground[:] = [ground[0], ground[1], ground[2], 1.0]
    c.jitter[:] = [0.0, 0.0, 1.0 if beauty else 0.0, footprint]
    c.ortho[:] = [1.0 if ortho else 0.0, max(np.tan(np.radians(contact_angle_deg)), 0.05), 0.0, 0.0]
    r = np.array([np.sin(yaw), -np.cos(yaw), 0.0])
    u = np.cross(r, (tgt - eye) / d)
    c.basis_r[:] = [r[0], r[1], r[2], 0.0]
    c.basis_u[:] = [u[0], u[1], u[2], 0.0]
    c.lens[:] = [lens[0], lens[1], lens[2], 1.0] if lens is not None else [0.0, 0.0, 0.0, 0.0]
    return c
