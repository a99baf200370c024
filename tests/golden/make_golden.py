"""Writes tests/golden/physics_kat.json: known answers the reference's own configuration derives with its own code
(configs/twin/physics.yaml in the reference project), read as text - no reference code is run:
  - materials.<name>.ior and .fresnel_avg "derived from ior" (gpu/bsdf.js:35 fresnelAverage, 4 decimals);
  - light.profile theta_deg / p and its projected_solid_angle "2 pi int p(theta) cos sin dtheta of the tabulated,
    linearly interpolated p" (gpu/shade_ref.js:5 profile);
  - light.profile's half-radiance note is not a number and is not used.
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
out = {"source": "configs/twin/physics.yaml (reference project), values derived there from the reference's own formulas",
       "fresnel_avg": pairs,
       "profile": {"theta_deg": json.loads(prof.group(1)), "p": json.loads(prof.group(2)), "projected_solid_angle": float(prof.group(3))}}
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "physics_kat.json")
json.dump(out, open(path, "w"), indent=1)
print(path, len(pairs), "fresnel pairs")
