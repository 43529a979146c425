"""CPU restatement of the volume ray-marching that LBM::render3d_* draws
(BoltzmannFluids/Source/LBM/LBM.cpp:1207-1376 with the fragment shaders
GLSL/Renderer3D/density_volumetric.frag, velocity_volumetric.frag,
boundries_volumetric.frag, forces_volumetric.frag,
temperature_volumetric.frag), for the product's headless CUDA renderer
(bf_render3d) to be checked against.  TEST INFRASTRUCTURE ONLY.

One ray per pixel from the camera through the pixel centre is clipped to the
unit cube [-0.5, 0.5]^3 and marched in steps of 1/sample_count while the
marched length is below the chord, sampling the fields at position + 0.5
with trilinear filtering (texel centres at (i + 1/2)/n, clamped to the edge);
each mode accumulates as its shader does.  Every step is one float32
operation in the kernel's order; exp is the Cody-Waite / Taylor exp_f32 of
the step kernels."""
import numpy as np

f32 = np.float32
DENSITY, VELOCITY, BOUNDRIES, FORCES, TEMPERATURE = range(5)


def exp_f32(x):
    x = f32(x)
    L2E, HI, LO = f32(float.fromhex("0x1.715476p+0")), f32(float.fromhex("0x1.62e4p-1")), f32(float.fromhex("0x1.7f7d1cp-20"))
    kf = f32(np.rint(f32(x * L2E)))
    r = f32(f32(x - f32(kf * HI)) - f32(kf * LO))
    q = f32(float.fromhex("0x1.a01a02p-13"))
    for c in ("0x1.6c16c2p-10", "0x1.111112p-7", "0x1.555556p-5", "0x1.555556p-3", "0x1p-1", "0x1p+0", "0x1p+0"):
        q = f32(f32(q * r) + f32(float.fromhex(c)))
    return f32(q * f32(np.ldexp(1.0, int(kf))))


def _sample(field, res, c, u, v, w):
    nx, ny, nz = res
    g = [f32(f32(u * f32(nx)) - f32(0.5)), f32(f32(v * f32(ny)) - f32(0.5)), f32(f32(w * f32(nz)) - f32(0.5))]
    fl = [f32(np.floor(x)) for x in g]
    t = [f32(g[k] - fl[k]) for k in range(3)]
    x0, y0, z0 = (int(x) for x in fl)

    def at(x, y, z):
        x = min(max(x, 0), nx - 1)
        y = min(max(y, 0), ny - 1)
        z = min(max(z, 0), nz - 1)
        return field[z, y, x, c]

    def lerp(a, b, s):
        return f32(a + f32(f32(b - a) * s))
    c00 = lerp(at(x0, y0, z0), at(x0 + 1, y0, z0), t[0])
    c10 = lerp(at(x0, y0 + 1, z0), at(x0 + 1, y0 + 1, z0), t[0])
    c01 = lerp(at(x0, y0, z0 + 1), at(x0 + 1, y0, z0 + 1), t[0])
    c11 = lerp(at(x0, y0 + 1, z0 + 1), at(x0 + 1, y0 + 1, z0 + 1), t[0])
    return lerp(lerp(c00, c10, t[1]), lerp(c01, c11, t[1]), t[2])


def _invert4(m):
    """Column-major 4x4 inverse by cofactors, the same double operations as the product's host code."""
    a = [0.0] * 16
    a[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10]
    a[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10]
    a[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9]
    a[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9]
    a[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10]
    a[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10]
    a[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9]
    a[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9]
    a[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6]
    a[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6]
    a[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5]
    a[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5]
    a[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6]
    a[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6]
    a[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5]
    a[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5]
    det = m[0] * a[0] + m[1] * a[4] + m[2] * a[8] + m[3] * a[12]
    return [x / det for x in a]


def camera_terms(view, projection):
    """(inverse(P V) as float32 column-major 16, camera position float32[3]); matrices column-major float32."""
    v = [float(x) for x in np.asarray(view, np.float32).reshape(-1)]
    pr = [float(x) for x in np.asarray(projection, np.float32).reshape(-1)]
    pv = [0.0] * 16
    for c in range(4):
        for row in range(4):
            acc = 0.0
            for k in range(4):
                acc += pr[k * 4 + row] * v[c * 4 + k]
            pv[c * 4 + row] = acc
    inv = _invert4(pv)
    vinv = _invert4(v)
    cam = np.array([vinv[12 + k] / vinv[15] for k in range(3)], np.float32)
    return np.array(inv, np.float32), cam


def render(vel_den, force_temp, bnd, res, mode, view, projection, width, height, samples, cam_terms=None):
    """vel_den/force_temp: (N, 4) float32, bnd: (N,) uint8 -> (height, width, 4) float32."""
    nx, ny, nz = res
    vd = np.asarray(vel_den, np.float32).reshape(nz, ny, nx, 4)
    ft = np.asarray(force_temp, np.float32).reshape(nz, ny, nx, 4)
    bd = (np.asarray(bnd, np.uint8).astype(np.float32) / f32(255)).astype(np.float32).reshape(nz, ny, nx, 1)
    m, cam = cam_terms if cam_terms is not None else camera_terms(view, projection)
    img = np.zeros((height, width, 4), np.float32)
    h = f32(f32(1) / f32(samples))
    for j in range(height):
        ndy = f32(f32(f32(2 * j + 1) / f32(height)) - f32(1))
        for i in range(width):
            ndx = f32(f32(f32(2 * i + 1) / f32(width)) - f32(1))
            r = [f32(f32(f32(f32(m[row] * ndx) + f32(m[4 + row] * ndy)) + f32(m[8 + row] * f32(1))) + m[12 + row])
                 for row in range(4)]
            far = [f32(r[k] / r[3]) for k in range(3)]
            d = [f32(far[k] - cam[k]) for k in range(3)]
            ln = f32(np.sqrt(f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2]))))
            if not ln > 0:
                continue
            d = [f32(x / ln) for x in d]
            tmin, tmax = f32(-np.inf), f32(np.inf)
            with np.errstate(divide="ignore", invalid="ignore"):
                for k in range(3):
                    inv = f32(f32(1) / d[k])
                    t0 = f32(f32(f32(-0.5) - cam[k]) * inv)
                    t1 = f32(f32(f32(0.5) - cam[k]) * inv)
                    tmin = max(tmin, min(t0, t1))
                    tmax = min(tmax, max(t0, t1))
            to_box = max(f32(0), tmin)
            in_box = max(f32(0), f32(tmax - to_box))
            if not in_box > 0:
                continue
            pos = [f32(cam[k] + f32(to_box * d[k])) for k in range(3)]
            depth, trans, hit = f32(0), f32(1), False
            acc = [f32(0)] * 3
            while depth < in_box:
                u, v, w = (f32(pos[k] + f32(0.5)) for k in range(3))
                if mode == DENSITY:
                    a = _sample(vd, res, 3, u, v, w)
                    trans = f32(trans * exp_f32(f32(f32(-a * f32(8)) * h)))
                    light = (f32(0.5), f32(0.8), f32(1.0))
                    acc = [f32(acc[k] + f32(f32(trans * light[k]) * h)) for k in range(3)]
                elif mode == VELOCITY:
                    for k in range(3):
                        s0 = _sample(vd, res, k, u, v, w)
                        s1 = _sample(vd, res, k, f32(f32(0.01) + u), f32(f32(0.01) + v), f32(f32(0.01) + w))
                        acc[k] = f32(acc[k] + f32(f32(abs(f32(s0 - s1)) * f32(32)) * h))
                elif mode == BOUNDRIES:
                    hit = hit or _sample(bd, res, 0, u, v, w) > 0
                elif mode == FORCES:
                    for k in range(3):
                        acc[k] = f32(acc[k] + f32(f32(abs(_sample(ft, res, k, u, v, w)) * f32(256)) * h))
                else:
                    acc[0] = f32(acc[0] + f32(_sample(ft, res, 3, u, v, w) * h))
                depth = f32(depth + h)
                pos = [f32(pos[k] + f32(d[k] * h)) for k in range(3)]
            if mode == DENSITY:
                a = f32(f32(1) - trans)
                img[j, i] = [f32(acc[0] / a), f32(acc[1] / a), f32(acc[2] / a), a]
            elif mode == VELOCITY:
                img[j, i] = [acc[0], acc[1], acc[2], acc[0]]
            elif mode == BOUNDRIES:
                img[j, i] = [1, 1, 1, 1 if hit else 0]
            elif mode == FORCES:
                r3 = [f32(f32(1) - exp_f32(-acc[k])) for k in range(3)]
                img[j, i] = [r3[0], r3[1], r3[2], r3[0]]
            else:
                img[j, i] = [1, 0, 0, acc[0]]
    return img


def look_at(eye, target, up=(0.0, 1.0, 0.0)):
    """Column-major view matrix (glm::lookAt)."""
    e, t, u = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = (t - e) / np.linalg.norm(t - e)
    s = np.cross(f, u); s /= np.linalg.norm(s)
    uu = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, uu, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ e, -uu @ e, f @ e
    return m.T.reshape(-1).astype(np.float32)


def perspective(fovy, aspect, near, far):
    """Column-major projection matrix (glm::perspective)."""
    t = np.tan(fovy / 2)
    m = np.zeros((4, 4))
    m[0, 0] = 1 / (aspect * t)
    m[1, 1] = 1 / t
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2 * far * near / (far - near)
    m[3, 2] = -1
    return m.T.reshape(-1).astype(np.float32)
