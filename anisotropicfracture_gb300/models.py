"""Per-node stiffness models, as coefficient arrays for ae_op_set_model.

Mirrors Model::Solid::Linear::{Isotropic, Cubic, Laplacian} and the E/nu conversion of
Model::Solid::Affine::Isotropic.  Coefficient layouts:
  ISOTROPIC  (lambda, mu)                     Set::Matrix4<3,Sym::Isotropic>  (src/Set/Matrix4_Isotropic.H:12-15)
  MAJORMINOR 21 slots                          Set::Matrix4<3,Sym::MajorMinor> (src/Set/Matrix4_MajorMinor.H:145-192)
  DIAGONAL   A(i,j) row-major                  Set::Matrix4<3,Sym::Diagonal>   (src/Set/Matrix4_Diagonal.H:117-126)
  MAJOR      45 slots: upper triangle of the 9 x 9 matrix A(3i+j, 3k+l), row by row
                                               Set::Matrix4<3,Sym::Major>      (src/Set/Matrix4_Major.H:203-258)
and the finite-kinematics Model::Solid::Elastic::NeoHookean, whose tangent is a MAJOR field.
"""
from dataclasses import dataclass

import numpy as np

ISOTROPIC, MAJORMINOR, DIAGONAL, MAJOR = 0, 1, 2, 3
NCOEF = {ISOTROPIC: 2, MAJORMINOR: 21, DIAGONAL: 9, MAJOR: 45}


@dataclass
class NeoHookean:
    """Model::Solid::Elastic::NeoHookean (src/Model/Solid/Elastic/NeoHookean.H:11-81): W(F) =
    mu/2 (F:F / |J|^(2/3) - 3) + kappa/2 (J - 1)^2 with kinematic variable F = I + grad u."""
    mu: float
    kappa: float


def major_slot(I, K):
    """Slot of entry (I, K) of the 9 x 9 matrix of a Sym::Major tensor."""
    if I > K:
        I, K = K, I
    return I * 9 - I * (I - 1) // 2 + (K - I)


def major_from_full(T):
    """45 Sym::Major slots of tensors shaped (..., 3, 3, 3, 3) (upper triangle of A(3i+j, 3k+l));
    returns (..., 45)."""
    A = np.asarray(T, dtype=np.float64).reshape(np.shape(T)[:-4] + (9, 9))
    rows, cols = np.triu_indices(9)
    return A[..., rows, cols]

# Voigt index of an index pair and the 21 storage slots of the reference's MajorMinor
# tensor, keyed by the (sorted) pair of Voigt indices: the table restates the uid map of
# src/Set/Matrix4_MajorMinor.H:148-189.
_VOIGT = np.array([[0, 5, 4], [5, 1, 3], [4, 3, 2]])
_SLOT_REPS = [((0, 0), (0, 0)), ((0, 0), (0, 1)), ((0, 0), (0, 2)), ((0, 0), (1, 1)), ((0, 0), (1, 2)),
              ((0, 0), (2, 2)), ((0, 1), (0, 1)), ((0, 1), (0, 2)), ((0, 1), (1, 1)), ((0, 1), (1, 2)),
              ((0, 1), (2, 2)), ((0, 2), (0, 2)), ((0, 2), (1, 1)), ((0, 2), (1, 2)), ((0, 2), (2, 2)),
              ((1, 1), (1, 1)), ((1, 1), (1, 2)), ((1, 1), (2, 2)), ((1, 2), (1, 2)), ((1, 2), (2, 2)),
              ((2, 2), (2, 2))]
SLOT = np.zeros((3, 3, 3, 3), dtype=np.int64)
_pair_slot = {}
for _s, (_a, _b) in enumerate(_SLOT_REPS):
    _va, _vb = _VOIGT[_a], _VOIGT[_b]
    _pair_slot[(_va, _vb)] = _s
    _pair_slot[(_vb, _va)] = _s
for _i in range(3):
    for _j in range(3):
        for _k in range(3):
            for _l in range(3):
                SLOT[_i, _j, _k, _l] = _pair_slot[(_VOIGT[_i, _j], _VOIGT[_k, _l])]


def lame_from_E_nu(E, nu):
    """src/Model/Solid/Affine/Isotropic.H:72-73"""
    E = np.asarray(E, dtype=np.float64)
    lam = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)
    mu = E / 2.0 / (1.0 + nu)
    return lam, mu


def isotropic(mu, lam):
    """Linear::Isotropic(mu, lambda) (src/Model/Solid/Linear/Isotropic.H:19-29) -> (lambda, mu)."""
    return np.array([lam, mu], dtype=np.float64)


def laplacian():
    """Linear::Laplacian: Diagonal tensor with A = ones (src/Model/Solid/Linear/Laplacian.H:31-34)."""
    return np.ones(9, dtype=np.float64)


def euler_rotation(phi1, Phi, phi2):
    """R = AngleAxis(phi2, X) * AngleAxis(Phi, Z) * AngleAxis(phi1, X)  (src/Model/Solid/Linear/Cubic.H:22-29)."""
    def rx(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])

    def rz(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    return rx(phi2) @ rz(Phi) @ rx(phi1)


def cubic_tensor(C11, C12, C44):
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    if i == j == k == l:
                        C[i, j, k, l] = C11
                    elif i == k and j == l:
                        C[i, j, k, l] = C44
                    elif i == j and k == l:
                        C[i, j, k, l] = C12
    return C


def cubic(C11, C12, C44, R):
    """Linear::Cubic::Define(C11, C12, C44, R): C'_pqst = R_pi R_qj R_sk R_tl C_ijkl stored in 21 slots
    (src/Model/Solid/Linear/Cubic.H:31-59).  R may be (3,3) or a stack (G,3,3); returns (21,) or (G,21).
    Each slot takes the value of the last (p,q,s,t), in loop order, that maps to it, as the reference's
    assignment loop does.  Each value is summed over (i,j,k,l) in the reference's loop order with the
    reference's product order, so the result equals the reference's bit for bit."""
    R = np.asarray(R, dtype=np.float64)
    single = R.ndim == 2
    R = R.reshape(-1, 3, 3)
    C = cubic_tensor(C11, C12, C44)
    last = {}
    for p in range(3):
        for q in range(3):
            for s in range(3):
                for t in range(3):
                    last[int(SLOT[p, q, s, t])] = (p, q, s, t)
    out = np.zeros((R.shape[0], 21))
    for slot, (p, q, s, t) in last.items():
        acc = np.zeros(R.shape[0])
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    for l in range(3):
                        acc = acc + R[:, p, i] * R[:, s, k] * C[i, j, k, l] * R[:, q, j] * R[:, t, l]
        out[:, slot] = acc
    return out[0] if single else out


def full_from_slots(c21):
    """81-entry tensor of a 21-slot MajorMinor tensor."""
    return np.asarray(c21)[..., SLOT]


def random_rotations(n, rng):
    """Haar-uniform rotations from uniform unit quaternions (Shoemake's method)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    w, x = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    y, z = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R
