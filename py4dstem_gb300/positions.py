"""Global affine constraint of corrected scan positions (host side).

With position correction and ``global_affine_transformation=True`` the reference
replaces the corrected positions, after every iteration, by the affine map of
the initial positions that best fits them (ptychographic_constraints.py:1313-1350):
a least-squares fit of a 3 x 2 matrix (two scales, a shear, a rotation and a
translation about the initial positions' centre of mass) on random subsets of
the positions drawn from NumPy's global random generator, refitted on the
consensus inliers, the best fit kept (RANSAC, utils.py:773-827). The fit is a
few 2 x 2 solves on float32 position arrays; it runs on the host between
iterations, with the same NumPy operations and random draws in the same order
as the reference, so the positions and the random sequence (which also shuffles
the batches) stay the reference's.
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class AffineTransform:
    """x -> (x - origin) @ (scale @ shear @ rotation) + (t0, t1) + origin
    (utils.py:580-741)."""

    scale0: float = 1.0
    scale1: float = 1.0
    shear1: float = 0.0
    angle: float = 0.0
    t0: float = 0.0
    t1: float = 0.0

    @classmethod
    def from_matrix(cls, T: np.ndarray) -> "AffineTransform":
        """Decompose a 2 x 2 (or 3 x 2 with the translation in its last row)
        matrix: Gram-Schmidt of the rows gives the scales and the shear, the
        remaining rotation its angle (the Graphics Gems II 7.1 method, in the
        reference's operation order)."""
        R = T[:2, :2].copy()
        s0 = np.linalg.norm(R[0])
        if s0 <= 0:
            return cls()
        R[0] /= s0
        sh = R[0] @ R[1]
        R[1] -= sh * R[0]
        s1 = np.linalg.norm(R[1])
        if s1 <= 0:
            return cls()
        R[1] /= s1
        sh /= s1
        angle = np.arccos(R[0, 0])
        t0, t1 = T[2] if T.shape[0] > 2 else (0.0, 0.0)
        return cls(scale0=float(s0), scale1=float(s1), shear1=float(sh), angle=float(angle),
                   t0=t0, t1=t1)

    def matrix(self) -> np.ndarray:
        """scale @ shear @ rotation as float32 2 x 2 matrices."""
        c = np.cos(self.angle)
        s = np.sin(self.angle)
        scale = np.array([[self.scale0, 0.0], [0.0, self.scale1]], dtype="float32")
        shear = np.array([[1.0, 0.0], [self.shear1, 1.0]], dtype="float32")
        rotation = np.array([[+c, -s], [+s, +c]], dtype="float32")
        return scale @ shear @ rotation

    def __call__(self, x: np.ndarray, origin=(0, 0)) -> np.ndarray:
        origin = np.asarray(origin, dtype=np.float32)
        m = np.asarray(self.matrix(), dtype=np.float32)
        shift = np.array((self.t0, self.t1)) + origin
        return ((x - origin) @ m) + shift


def fit_affine(positions0, positions1, origin=(0, 0), translation=True):
    """Least-squares affine map of positions0 onto positions1 about `origin`
    (normal equations), and the L2 norm of its residual (utils.py:743-770)."""
    origin = np.asarray(origin, dtype=np.float32)
    try:
        a = positions0 - origin
        if translation:
            a = np.pad(a, ((0, 0), (0, 1)), constant_values=1)
        b = positions1 - origin
        at = a.conj().swapaxes(-1, -2)
        tf = AffineTransform.from_matrix(np.linalg.inv(at @ a) @ at @ b)
    except np.linalg.LinAlgError:
        tf = AffineTransform()
    return tf, np.linalg.norm(tf(positions0, origin=origin) - positions1)


def fit_affine_ransac(positions0, positions1, origin=(0, 0), translation=True,
                      min_sample=64, max_error=16, min_consensus=0.75, max_iter=20):
    """Best consensus fit over `max_iter` random subsets of `min_sample` indices
    (drawn with replacement from NumPy's global generator in one call); a
    subset whose fit leaves at least `min_consensus` of the positions within
    `max_error` pixels is refitted on those, the smallest residual kept
    (utils.py:773-827)."""
    best = np.inf
    transform = AffineTransform()
    for subset in np.random.choice(a=len(positions0), size=(max_iter, min_sample),
                                   replace=True):
        subset = np.unique(subset)
        model, _ = fit_affine(positions0[subset], positions1[subset], origin, translation)
        dist = np.linalg.norm(model(positions0, origin=origin) - positions1, axis=-1)
        inliers = dist <= max_error
        if np.sum(inliers) / len(inliers) >= min_consensus:
            model, fitness = fit_affine(positions0[inliers], positions1[inliers], origin,
                                        translation)
            if fitness < best:
                best = fitness
                transform = model
    return transform, best


def affine_constraint(initial_positions: np.ndarray, current_positions: np.ndarray):
    """(constrained positions, transform): the RANSAC affine map of the initial
    positions onto the current ones, applied to the initial positions
    (ptychographic_constraints.py:1313-1350; subsets of a tenth of the scan)."""
    com = initial_positions.mean(0)
    tf, _ = fit_affine_ransac(initial_positions, current_positions, origin=com,
                              translation=True, min_sample=initial_positions.shape[0] // 10)
    return tf(initial_positions, origin=com), tf
