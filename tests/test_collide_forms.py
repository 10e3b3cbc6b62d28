"""The moment form of the regularized + Smagorinsky collision that the f16 / bf16
step kernels run on scaled deviations (collide_dev in wt_lbm.cu), transcribed in
float64, against the textbook form the reference writes out (wgsl.ts:231-272:
feq from rho and u, Pi^neq = sum (f - feq) c c, f' = feq + (1 - 1/tau) 4.5 w
(c c - I/3) : Pi^neq) on random states near equilibrium: the two agree to
float64 round-off, so the f16 / bf16 kernels differ from the reference only by
FP32 rounding."""
import numpy as np

C = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0], [-1, -1, 0],
              [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1], [0, 1, 1], [0, -1, -1],
              [0, 1, -1], [0, -1, 1]], float)
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def textbook(f, tau0, ks2):
    rho = f.sum()
    u = (f[:, None] * C).sum(0) / rho
    cu = C @ u
    feq = W * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u @ u)
    pi = np.einsum("i,ia,ib->ab", f - feq, C, C)
    q = np.sqrt((pi * pi).sum())
    tau = 0.5 * (tau0 + np.sqrt(tau0 * tau0 + ks2 * q / rho))
    qi = np.einsum("ia,ib,ab->i", C, C, pi) - np.trace(pi) / 3
    return feq + (1 - 1 / tau) * 4.5 * W * qi


def moment_form(d, tau0, ks2, S):
    """collide_dev's steps in float64: d = S (f - w) in, S (f' - w) out."""
    s = d[1::2] + d[2::2]
    m = d[1::2] - d[2::2]
    jx = m[0] + m[3] + m[4] + m[5] + m[6]
    jy = m[1] + m[3] - m[4] + m[7] + m[8]
    jz = m[2] + m[5] - m[6] + m[7] - m[8]
    sxx = s[0] + s[3] + s[4] + s[5] + s[6]
    syy = s[1] + s[3] + s[4] + s[7] + s[8]
    szz = s[2] + s[5] + s[6] + s[7] + s[8]
    sxy, sxz, syz = s[3] - s[4], s[5] - s[6], s[7] - s[8]
    dr = (d[0] + s.sum()) / S
    rho = 1 + dr
    ux, uy, uz = jx / S / rho, jy / S / rho, jz / S / rho
    uu = ux * ux + uy * uy + uz * uz
    pxx = sxx / S - rho * ux * ux - dr / 3
    pyy = syy / S - rho * uy * uy - dr / 3
    pzz = szz / S - rho * uz * uz - dr / 3
    pxy, pxz, pyz = sxy / S - rho * ux * uy, sxz / S - rho * ux * uz, syz / S - rho * uy * uz
    qn = np.sqrt(pxx ** 2 + pyy ** 2 + pzz ** 2 + 2 * (pxy ** 2 + pxz ** 2 + pyz ** 2))
    tau = 0.5 * (tau0 + np.sqrt(tau0 * tau0 + ks2 * qn / rho))
    k = 4.5 * (1 - 1 / tau)
    tr3 = (pxx + pyy + pzz) / 3
    a = dr - 1.5 * rho * uu
    qx, qy, qz = pxx - tr3, pyy - tr3, pzz - tr3
    bxy, bxz, byz = qx + pyy, qx + pzz, qy + pzz
    qd = [qx, qy, qz, bxy + 2 * pxy, bxy - 2 * pxy, bxz + 2 * pxz, bxz - 2 * pxz, byz + 2 * pyz, byz - 2 * pyz]
    out = np.zeros(19)
    out[0] = S * W[0] * (a - k * tr3)
    u = np.array([ux, uy, uz])
    for p in range(9):
        i = 2 * p + 1
        cu = C[i] @ u
        e = a + k * qd[p] + 4.5 * rho * cu * cu
        out[i] = S * W[i] * (e + 3 * rho * cu)
        out[i + 1] = S * W[i] * (e - 3 * rho * cu)
    return out


def test_moment_form_equals_textbook():
    rng = np.random.default_rng(0)
    ks2 = 18 * 1.41421356 * 0.1 ** 2
    for S in (16384.0, 1.0):
        for _ in range(200):
            rho = 1 + rng.uniform(-0.05, 0.05)
            u = rng.uniform(-0.12, 0.12, 3)
            cu = C @ u
            f = W * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u @ u) + rng.normal(0, 2e-3, 19) * W
            tau0 = rng.uniform(0.505, 0.9)
            want = (textbook(f, tau0, ks2) - W) * S
            got = moment_form((f - W) * S, tau0, ks2, S)
            np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12 * S)
