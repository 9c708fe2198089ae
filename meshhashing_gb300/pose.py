"""se(3) helpers for the differentiable raycast (host side, double precision).

Pose increments are left increments of the camera-to-world pose,
wTc <- exp(xi) wTc, with xi = (tx, ty, tz, wx, wy, wz): translation first,
then rotation, as mh_raycast_backward and mh_refine_pose use them.
"""
from __future__ import annotations

import numpy as np


def hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def se3_exp(xi) -> np.ndarray:
    xi = np.asarray(xi, np.float64)
    u, w = xi[:3], xi[3:]
    th = float(np.linalg.norm(w))
    W = hat(w)
    if th < 1e-5:
        A, B, C = 1.0 - th * th / 6.0, 0.5 - th * th / 24.0, 1.0 / 6.0 - th * th / 120.0
    else:
        A, B, C = np.sin(th) / th, (1.0 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
    R = np.eye(3) + A * W + B * W @ W
    V = np.eye(3) + B * W + C * W @ W
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = V @ u
    return T


def se3_log(T) -> np.ndarray:
    T = np.asarray(T, np.float64)
    R, t = T[:3, :3], T[:3, 3]
    c = np.clip((np.trace(R) - 1.0) / 2.0, -1.0, 1.0)
    th = float(np.arccos(c))
    if th < 1e-8:
        w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
    else:
        w = th / (2.0 * np.sin(th)) * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    W = hat(w)
    th = float(np.linalg.norm(w))
    if th < 1e-5:
        Vinv = np.eye(3) - 0.5 * W + W @ W / 12.0
    else:
        Vinv = np.eye(3) - 0.5 * W + (1.0 / th ** 2) * (1.0 - (th * np.sin(th)) / (2.0 * (1.0 - np.cos(th)))) * W @ W
    return np.concatenate([Vinv @ t, w])


def left_update(wTc, xi) -> np.ndarray:
    """exp(xi) @ wTc."""
    return se3_exp(xi) @ np.asarray(wTc, np.float64)


def pose_error(T_est, T_ref):
    """(translation error in metres, rotation error in degrees)."""
    D = np.linalg.inv(np.asarray(T_ref, np.float64)) @ np.asarray(T_est, np.float64)
    c = np.clip((np.trace(D[:3, :3]) - 1.0) / 2.0, -1.0, 1.0)
    return float(np.linalg.norm(np.asarray(T_est)[:3, 3] - np.asarray(T_ref)[:3, 3])), float(np.degrees(np.arccos(c)))
