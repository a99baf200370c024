"""Writes tests/golden/physics_kat.json: known answers the reference's own configuration derives with its own code
(configs/twin/physics.yaml in the reference project), read as text - no reference code is run:
  - materials.<name>.ior and .fresnel_avg "derived from ior" (gpu/bsdf.js:35 fresnelAverage, 4 decimals);
  - light.profile theta_deg / p and its projected_solid_angle "2 pi int p(theta) cos sin dtheta of the tabulated,
    linearly interpolated p" (gpu/shade_ref.js:5 profile);
  - light.profile's half-radiance note is not a number and is not used;
  - materials whose rho_d is "derived: albedo / (1 - F0), F0 = ...": albedo, rho_d, ior and the stated F0;
  - the light outlet's area_on_face and area_cross_section, flux_at_scope_tip, srgb_chromaticity and the emitter's L0
    (L0 = Y0 x chromaticity, Y0 = flux / (683 A_face int p cos dw)).
Run beside a checkout of the reference (../reference from this repository, or $VT_REFERENCE), or pass its path:
python make_golden.py /path/to/reference
"""
import json
import os
import re
import sys

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VT_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
text = open(os.path.join(ref, "configs", "twin", "physics.yaml")).read()
val = lambda s: json.loads(s) if s.strip().startswith("[") else float(s)

pairs = []
cur = None
for line in text.splitlines():
    m = re.match(r"^  ([a-z_]+):\s*$", line)
    if m:
        cur = {"name": m.group(1)}
        continue
    m = re.match(r"^    (ior|fresnel_avg): \{value: ([-0-9.e+]+),", line)
    if m and cur is not None:
        cur[m.group(1)] = float(m.group(2))
        if m.group(1) == "fresnel_avg" and "ior" in cur and "derived from ior" in line:
            pairs.append({"name": cur["name"], "ior": cur["ior"], "fresnel_avg": cur["fresnel_avg"]})
prof = re.search(r"  profile:\n(?:.*\n)*?    theta_deg: \{value: (\[[^\]]*\])(?:.*\n)*?    p: \{value: (\[[^\]]*\])(?:.*\n)*?    projected_solid_angle: \{value: ([0-9.]+)", text)
# materials whose rho_d is "derived: albedo / (1 - F0), F0 = ..." (F0 the normal-incidence Fresnel of their ior)
derived = []
cur = None
for line in text.splitlines():
    m = re.match(r"^  ([a-z_]+):\s*$", line)
    if m:
        cur = {"name": m.group(1)}
        continue
    if cur is None:
        continue
    m = re.match(r"^    (albedo|rho_d|ior): \{value: (\[[^\]]*\]|[-0-9.e+]+),(.*)$", line)
    if m:
        cur[m.group(1)] = val(m.group(2))
        f = re.search(r"albedo / \(1 - F0\), F0 = ([0-9.]+)", m.group(3))
        if m.group(1) == "rho_d" and f:
            cur["F0"] = float(f.group(1))
    if {"albedo", "rho_d", "ior", "F0"} <= set(cur) and cur not in derived:
        derived.append(cur)
num = lambda key: float(re.search(r"\n\s*" + key + r": \{value: ([-0-9.e+]+)", text).group(1))
vec = lambda key: json.loads(re.search(r"\n\s*" + key + r": \{value: (\[[^\]]*\])", text).group(1))
light = {"area_on_face": num("area_on_face"), "area_cross_section": num("area_cross_section"), "flux_lm": num("flux_at_scope_tip"),
         "srgb_chromaticity": vec("srgb_chromaticity"), "L0": vec("L0"),
         "note": "L0 = Y0 x srgb_chromaticity with Y0 = flux / (683 A_face int p cos dw) (physics.yaml materials.emitter.L0); "
                 "area_on_face = area_cross_section / cos 30 deg, Monte-Carlo check 4.790e-5"}
out = {"source": "configs/twin/physics.yaml (reference project), values derived there from the reference's own formulas",
       "fresnel_avg": pairs,
       "profile": {"theta_deg": json.loads(prof.group(1)), "p": json.loads(prof.group(2)), "projected_solid_angle": float(prof.group(3))},
       "rho_d_from_albedo": [{k: d[k] for k in ("name", "albedo", "rho_d", "ior", "F0")} for d in derived],
       "light": light}
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "physics_kat.json")
json.dump(out, open(path, "w"), indent=1)
print(path, len(pairs), "fresnel pairs")
