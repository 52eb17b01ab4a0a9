"""Generate tests/golden/hertz_collision_time.json: the analytic Hertz collision times of the
reference's known-answer test py/tests/hertz.py:29-46 (two spheres r=0.05 m, rho=1e3, E=1e8,
nu=0.2, impact velocities 1 .. 1e-5 m/s): tau = 2.214 (rho/E*)^(2/5) d v0^(-1/5)."""
import json
import os

r, rho, E, nu = 0.05, 1e3, 1e8, 0.2
Eeff = (E * E) / (E * (1 - nu ** 2) + E * (1 - nu ** 2))
d = 2 * r
out = {"source": "py/tests/hertz.py:29-46", "rho": rho, "Eeff": Eeff, "d": d, "tau": {}}
for v0 in (1, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
    out["tau"][str(v0)] = 2.214 * (rho / Eeff) ** (2 / 5.) * (d / v0 ** (1 / 5.))
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "hertz_collision_time.json"), "w") as f:
    json.dump(out, f, indent=1)
