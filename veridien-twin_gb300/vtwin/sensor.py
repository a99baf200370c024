"""gpu/sensor.js host logic: sensor parameters with defaults (sensorParams), the 256-byte sensor uniform
(packSensorUniform), the modelled raw noise and the analogue-gain map. The GPU stage itself is libvtwin's
sensor-expose kernel."""
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


def analog_gain(p: dict, uvc_gain: float, gain_range=(0, 100)) -> float:
    """gpu/sensor.js:93 analogGain: UVC gain units -> linear analogue gain."""
    g0, g1 = gain_range
    return 1 + (min(g1, max(g0, uvc_gain)) - g0) / max(1, g1 - g0) * (p["analogGainMax"] - 1)
