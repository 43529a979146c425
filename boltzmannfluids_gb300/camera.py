"""Camera matrices for render3d: column-major 4x4 float32 arrays laid out
as glm::lookAt and glm::perspective return them (the reference's Camera
hands these to LBM::render3d_*, LBM.cpp:1207-1376)."""
import numpy as np


def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    """View matrix looking from `eye` at `target`."""
    e, t, u = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = (t - e) / np.linalg.norm(t - e)
    s = np.cross(f, u)
    s /= np.linalg.norm(s)
    v = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, v, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ e, -v @ e, f @ e
    return m.T.reshape(-1).astype(np.float32)


def perspective(fovy, aspect, near, far):
    """Projection matrix: vertical field of view `fovy` (radians)."""
    t = np.tan(fovy / 2)
    m = np.zeros((4, 4))
    m[0, 0] = 1 / (aspect * t)
    m[1, 1] = 1 / t
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2 * far * near / (far - near)
    m[3, 2] = -1
    return m.T.reshape(-1).astype(np.float32)
