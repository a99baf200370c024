"""gpu/sensor.js host logic: sensor parameters with defaults (sensorParams), the 256-byte sensor uniform
(packSensorUniform), the modelled raw noise, the analogue-gain map, the UVC-style auto exposure and the grey-world
auto white balance. The GPU stages are libvtwin's sensor chain (vt_sensor_frame) and expose stage."""
from __future__ import annotations

import math
import struct

import numpy as np

CFA = {"RGGB": 0, "GRBG": 1, "GBRG": 2, "BGGR": 3}
_H, _C = 6.62607015e-34, 299792458.0
CHANNEL_NM = (600, 540, 460)


def sensor_params(over: dict | None = None) -> dict:
    """gpu/sensor.js:17 sensorParams with the physics-free defaults; `over` overrides any field."""
    pitch, qe = 3e-6, (0.45, 0.55, 0.5)
    g = [pitch * pitch * qe[c] * (nm * 1e-9) / (_H * _C) for c, nm in enumerate(CHANNEL_NM)]
    p = {
        "responseMatrix": [[g[0], 0, 0], [0, g[1], 0], [0, 0, g[2]]], "fNumber": 2.0, "transmission": 0.9,
        "esfSigmaPx": 0.7, "esfIncludesAperture": True, "readNoise": 3.0, "fullWell": 10000.0, "darkCurrent": 0.0,
        "conversionGain": 0.33, "adcBits": 12, "blackLevel": 0.0, "cfa": "GRBG", "wb": [1, 1, 1],
        "ccm": [[1, 0, 0], [0, 1, 0], [0, 0, 1]], "tone": "srgb", "sCurveC": None, "blackOffset": 0.0,
        "demosaic": "bilinear", "noiseReduction": "none", "nrSigmaPx": 0.4, "nrRangeScale": 2.0,
        "glareFraction": 0.0, "glareSigmaFrac": 0.25, "glareLevel": 16, "gamma": 2.2, "sharpenAmount": 0.0,
        "sharpenRadius": 1.0, "chroma": "4:2:0", "noise": True, "analogGainMax": 8.0,
        "pupilExponent": 1.0, "vignettingThetaDeg": [0.0, 90.0], "vignetting": [1.0, 1.0],
        "exposureUnit": 1e-4, "exposureRange": [1, 5000], "gainRange": [0, 100], "fps": 20, "aeTarget": 0.45,
        "aeDamping": 0.3, "aeMaxStep": 2.0, "awb": True, "awbDamping": 0.3, "exposureUnits0": 10,
    }
    p.update(over or {})
    return p


def unit_radiance_sensor(electrons_per_unit=4.0, read_noise=2.0, bits=12, cfa="RGGB") -> dict:
    """The batched configuration's sensor: RGGB Bayer, `electrons_per_unit` e- per unit radiance, read noise
    sigma, `bits`-bit ADC at 1 DN per e-, no optics blur, no glare, no full-well clip below the ADC range."""
    e = electrons_per_unit
    return sensor_params({"responseMatrix": [[e, 0, 0], [0, e, 0], [0, 0, e]], "esfSigmaPx": 0.0, "esfIncludesAperture": False,
                          "readNoise": read_noise, "fullWell": 1e9, "darkCurrent": 0.0, "conversionGain": 1.0,
                          "adcBits": bits, "blackLevel": 0.0, "cfa": cfa, "glareFraction": 0.0})


def pack_sensor_uniform(p: dict, width: int, height: int, frame=0, seed=0, exposure=1.0, gain=1.0, cam_index=0) -> np.ndarray:
    """gpu/sensor.js:158 packSensorUniform: 64 32-bit words (float and uint views of one buffer)."""
    buf = bytearray(256)
    f = lambda i, v: struct.pack_into("<f", buf, 4 * i, float(v))
    u = lambda i, v: struct.pack_into("<I", buf, 4 * i, int(v) & 0xFFFFFFFF)
    u(0, width); u(1, height); u(2, CFA.get(p["cfa"], 1)); u(3, frame)
    s_opt = math.sqrt(max(0.0, p["esfSigmaPx"] ** 2 - 1 / 12)) if p["esfIncludesAperture"] else p["esfSigmaPx"]
    f(4, math.pi * p["transmission"] / (4 * p["fNumber"] ** 2)); f(5, s_opt); f(6, exposure); f(7, gain)
    for r in range(3):
        for c in range(3):
            f(8 + 4 * r + c, p["responseMatrix"][r][c])
    f(20, p["readNoise"]); f(21, p["fullWell"]); f(22, p["darkCurrent"]); f(23, p["conversionGain"])
    f(24, 2 ** p["adcBits"] - 1); f(25, p["blackLevel"]); u(26, seed); f(27, 1 if p["noise"] else 0)
    f(28, p["wb"][0]); f(29, p["wb"][1]); f(30, p["wb"][2])
    for r in range(3):
        for c in range(3):
            f(32 + 4 * r + c, p["ccm"][r][c])
    tone = p["tone"]
    f(44, (3 if p["sCurveC"] else 0) if tone == "srgb" else (2 if tone == "linear" else 1))
    f(45, p["gamma"]); f(46, p["sharpenAmount"]); f(47, p["sharpenRadius"])
    u(48, 1 if str(p["chroma"]).startswith("4:2:0") else 0); u(49, cam_index)
    dm = str(p["demosaic"]).lower()
    u(50, 2 if "hamilton" in dm else 1 if "edge" in dm else 0)
    nr = str(p["noiseReduction"])
    u(51, 1 if any(k in nr for k in ("edge", "bilateral", "on")) else 0)
    F = p["glareLevel"] or 16
    f(52, p["glareFraction"] or 0); f(53, p["glareSigmaFrac"] * math.hypot(width, height) / F); f(54, F)
    f(56, p["sCurveC"] or 1); f(57, p["blackOffset"] or 0); f(58, p["nrSigmaPx"] or 0); f(59, p["nrRangeScale"] or 2)
    return np.frombuffer(bytes(buf), np.uint32).copy()


def raw_noise_dn(p: dict, e: float, gain: float) -> float:
    """gpu/sensor.js:180 rawNoiseDN: modelled raw noise std (DN) at a mean of e electrons."""
    return math.sqrt(max(0.0, e) + p["readNoise"] ** 2) * p["conversionGain"] * gain


def analog_gain(p: dict, uvc_gain: float, gain_range=None) -> float:
    """gpu/sensor.js:93 analogGain: UVC gain units -> linear analogue gain."""
    g0, g1 = gain_range or p.get("gainRange", (0, 100))
    return 1 + (min(g1, max(g0, uvc_gain)) - g0) / max(1, g1 - g0) * (p["analogGainMax"] - 1)


class AutoExposure:
    """gpu/sensor.js:128 AutoExposure: exposure time first (whole exposure units, up to the frame time), then
    analogue gain, damped toward the target mean luma; fed the previous frame's mean output luma."""

    def __init__(self, p: dict, exposure_units=10, gain_units=0, enabled=True):
        self.p, self.units, self.gain_units, self.enabled = p, exposure_units, gain_units, enabled
        self.product = self.units * p["exposureUnit"] * analog_gain(p, gain_units)

    @property
    def exposure(self) -> float:
        return self.units * self.p["exposureUnit"]

    @property
    def gain(self) -> float:
        return analog_gain(self.p, self.gain_units)

    def update(self, mean_luma: float) -> dict:
        if not self.enabled:
            return {"exposure": self.exposure, "gain": self.gain}
        p = self.p
        gam = 1.0 if p["tone"] == "linear" else 2.2
        ratio = (p["aeTarget"] / mean_luma) ** gam if mean_luma > 1e-4 else 8.0
        ratio = min(8.0, max(1 / 8, ratio))
        ms = p.get("aeMaxStep") or 2.0
        step = min(ms, max(1 / ms, ratio ** p["aeDamping"]))
        self.product *= step
        unit = p["exposureUnit"]
        max_units = min(p["exposureRange"][1], math.floor(1 / (p["fps"] * unit)))
        want = self.product / unit
        self.units = max(p["exposureRange"][0], min(max_units, _js_round(want)))
        g = self.product / (self.units * unit)
        g0, g1 = p["gainRange"]
        gu = g0 + (max(1.0, min(p["analogGainMax"], g)) - 1) / (p["analogGainMax"] - 1) * (g1 - g0)
        self.gain_units = _js_round(gu)
        self.product = max(p["exposureRange"][0] * unit, min(max_units * unit * p["analogGainMax"], self.product))
        return {"exposure": self.exposure, "gain": self.gain}


def _js_round(x: float) -> int:
    """JavaScript Math.round: halves go up."""
    return int(math.floor(x + 0.5))


def update_awb(prev, mean_rgb, damping=0.3):
    """gpu/sensor.js:184 updateAWB: grey-world gains equalising the raw channel means, damped in the log domain."""
    g = list(prev) if prev is not None else [1.0, 1.0, 1.0]
    if not (mean_rgb[0] > 1e-4 and mean_rgb[1] > 1e-4 and mean_rgb[2] > 1e-4):
        return g
    target = [mean_rgb[1] / mean_rgb[0], 1.0, mean_rgb[1] / mean_rgb[2]]
    return [math.exp(math.log(x) + damping * (math.log(target[c]) - math.log(x))) for c, x in enumerate(g)]
