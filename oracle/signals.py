"""Input signal and material helpers (FP64) - oracle only."""
import numpy as np


def gaussian_pulse(t, centre_freq, no_cycles):
    """fn_gaussian_pulse.m:1-15 (-40 dB Gaussian toneburst, shifted to start
    at the first sample whose envelope exceeds 0.01)."""
    t = np.asarray(t, float)
    sz = t.shape
    t = t.ravel()
    beta = 0.01
    ct = t.mean()
    T = no_cycles / (2 * centre_freq * np.sqrt(np.log(1 / beta)))
    env = np.exp(-((t - ct) / T) ** 2)
    i = np.nonzero(env > 0.01)[0].min()
    s = env * np.sin(2 * np.pi * centre_freq * (t - ct))
    s = np.concatenate([s[i:], np.zeros(i)])
    return s.reshape(sz)


def isotropic_stiffness_matrix(E, v):
    """fn_isotropic_stiffness_matrix.m:17-23 (6x6, engineering shear)."""
    g = (1 - 2 * v) / 2
    D = np.array([[1 - v, v, v, 0, 0, 0],
                  [v, 1 - v, v, 0, 0, 0],
                  [v, v, 1 - v, 0, 0, 0],
                  [0, 0, 0, g, 0, 0],
                  [0, 0, 0, 0, g, 0],
                  [0, 0, 0, 0, 0, g]], float)
    return E / (1 - 2 * v) / (1 + v) * D


def estimate_max_min_vels(matls):
    """fn_estimate_max_min_vels.m:1-28."""
    v = []
    for mt in matls:
        s = np.asarray(mt["D"], float).ravel()
        rho = mt["density"] if "density" in mt else mt["rho"]
        s = s[np.abs(s) > 0]
        if s.size:
            v.append((np.sqrt(s.min() / rho), np.sqrt(s.max() / rho)))
    v = np.array(v)
    return v[:, 1].max(), v[:, 0].min()


def get_suitable_time_step(matls, el_size, safety_factor=np.sqrt(2)):
    """fn_get_suitable_time_step.m:1-17."""
    mx, _ = estimate_max_min_vels(matls)
    return el_size / mx / safety_factor


def get_suitable_el_size(matls, centre_freq, els_per_wavelength):
    """fn_get_suitable_el_size.m:1-12."""
    _, mn = estimate_max_min_vels(matls)
    return mn / centre_freq / els_per_wavelength


def element_eigen_time_step(nds, els, D, rho, factor=0.9):
    """Stable step from the largest element eigenvalue of M_e^-1 K_e.

    The benchmark configurations ask for dt = factor * 2 / sqrt(lambda_max)
    over all CPE3 elements; FP64 dense eigenvalues per element.
    """
    from .elements import el_CPE3
    K, _, M, _, _ = el_CPE3(nds, els, D, rho, [1, 2])
    m = np.einsum("eii->ei", M)
    # symmetric scaling M^-1/2 K M^-1/2; the sign keeps clockwise elements
    # (negative detJ, so negative K and M) positive semi-definite
    A = K * np.sign(m[:, :, None]) / np.sqrt(np.abs(m[:, :, None] * m[:, None, :]))
    lam = np.linalg.eigvalsh(A).max()
    return factor * 2.0 / np.sqrt(lam)
