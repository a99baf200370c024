"""Twin calibration as an autograd-style function of one flat parameter vector.

    x = [albedo (n_materials x 3), lamp radiance (n_lamps), KB4 intrinsics (n_cameras x 8: fx, fy, cx, cy, k1..k4)]
    loss(x) = image loss (mean over pixels and channels of (I - T)^2, vt_calib_forward)
              + w_reproj x reprojection loss (mean over cameras, fiducials and both coordinates, vt_reproj_loss)

`Calibration.forward(x)` returns the loss and keeps what `backward()` needs; `backward()` returns d loss / d x:
the albedo and lamp entries by path replay and the transposed radiosity solve (vt_calib_backward); the intrinsics
by the reprojection term's analytic KB4 Jacobian and, with image_intrinsics=True, the image term's derivative along
every path's primary ray (vt_calib_intrinsics_grad: hit points, normals, light samples' weights, continuations,
through the KB4 inverse). The image term's steps (a ray's hit triangle, a shadow ray's outcome) are not
differentiated, and with intrinsics far from the target's (10 %: edges tens of pixels apart) those steps carry most
of the image loss's dependence on K, so by default the intrinsics follow the fiducials alone.
"""
from __future__ import annotations

import numpy as np


class Calibration:
    def __init__(self, renderer, cameras, targets, fiducials=None, uv_targets=None, w_reproj=1.0, spp=32, light_samples=1, seed=0,
                 max_depth=3, jacobi_iters=0, image_intrinsics=False):
        self.r = renderer
        self.cameras = [renderer._cam(c) for c in cameras]
        self.targets = [np.ascontiguousarray(t, np.float32) for t in targets]
        self.fid = None if fiducials is None else np.ascontiguousarray(fiducials, np.float64)
        self.uv_t = None if uv_targets is None else np.ascontiguousarray(uv_targets, np.float64)
        self.w = float(w_reproj)
        self.kw = dict(spp=spp, lightSamples=light_samples, seed=seed, max_depth=max_depth, jacobi_iters=jacobi_iters,
                       intrinsics=bool(image_intrinsics))
        self.image_intrinsics = bool(image_intrinsics)
        info = renderer.calib_info
        self.n_mat, self.n_lamps = info["n_materials"], info["n_lamps"]
        self.n = 3 * self.n_mat + self.n_lamps + 8 * len(self.cameras)
        self._last = None

    # ------------------------------------------------------------------------------------------ packing
    def pack(self, albedo, lamp, intrinsics) -> np.ndarray:
        return np.concatenate([np.asarray(albedo, np.float64).ravel(), np.asarray(lamp, np.float64).ravel(),
                               np.asarray(intrinsics, np.float64).ravel()])

    def unpack(self, x):
        x = np.asarray(x, np.float64)
        a = x[:3 * self.n_mat].reshape(self.n_mat, 3)
        l = x[3 * self.n_mat:3 * self.n_mat + self.n_lamps]
        K = x[3 * self.n_mat + self.n_lamps:].reshape(len(self.cameras), 8)
        return a, l, K

    def current(self) -> np.ndarray:
        """The renderer's intrinsics as a parameter vector tail (albedo and lamp parts zero)."""
        K = np.stack([self.r.get_intrinsics(c) for c in self.cameras])
        return self.pack(np.zeros((self.n_mat, 3)), np.zeros(self.n_lamps), K)

    # ------------------------------------------------------------------------------------------ the pair
    def forward(self, x) -> float:
        a, l, K = self.unpack(x)
        for c, k in zip(self.cameras, K):
            self.r.set_intrinsics(c, k)
        img, _ = self.r.calib_forward(self.cameras, a, l, targets=self.targets, images=False, **self.kw)
        rep, gK = 0.0, np.zeros((len(self.cameras), 8))
        if self.fid is not None:
            rep, gK = self.r.reproj_loss(self.cameras, self.fid, self.uv_t)
        self._last = (gK,)
        self.parts = {"image": img, "reproj": rep}
        return img + self.w * rep

    def backward(self) -> np.ndarray:
        if self._last is None:
            raise RuntimeError("backward before forward")
        (gK,) = self._last
        ga, gl = self.r.calib_backward()
        gi = self.r.calib_intrinsics_grad() if self.image_intrinsics else 0.0
        return self.pack(ga, gl, gi + self.w * gK)

    def loss_and_grad(self, x):
        f = self.forward(x)
        return f, self.backward()

