"""Per-field comparison of two runs of the same scene, matched by particle id.

Both runs keep their particles in their own cell-sorted order, so fields are gathered by
``id0`` (the upload index, eng/particle_system.py:208-211) before they are compared.
Errors are computed on the device in f64:

* ``max_rel`` / ``rms_rel`` - |a - b| / |b| per particle, for fields that stay away from
  zero (density);
* ``max_norm`` / ``rms_norm`` - |a - b| / max |b| (vector fields use the Euclidean norm
  per particle), for fields that pass through zero (pressure, velocity, rates, stress);
* ``max_abs`` - largest |a - b| (positions, in metres).

Only the particles selected by ``mask`` ("flow": fluid and soil, the default; "all")
enter the statistics.
"""
import torch

FIELDS = ("density", "pressure", "v", "x", "d_density", "d_vel")
KINDS = {"density": "rel", "x": "abs"}


def _ordered(ps, name):
    t = ps.field(name)
    order = torch.argsort(ps.field("id0").long())
    return t[order].to(torch.float64)


def field_errors(ps_a, ps_b, fields=FIELDS, mask="flow"):
    """Error of run a against run b (the reference run) for each named field."""
    mt = _ordered(ps_b, "mat_type")
    sel = (mt > 0) if mask == "flow" else torch.ones_like(mt, dtype=torch.bool)
    out = {}
    for name in fields:
        try:
            a, b = _ordered(ps_a, name), _ordered(ps_b, name)
        except Exception:  # a field one form does not export (e.g. stress of a WC scene)
            continue
        a, b = a[sel], b[sel]
        if a.dim() > 1:
            a, b = a.reshape(a.shape[0], -1), b.reshape(b.shape[0], -1)
            diff, ref = torch.linalg.vector_norm(a - b, dim=1), torch.linalg.vector_norm(b, dim=1)
        else:
            diff, ref = (a - b).abs(), b.abs()
        if diff.numel() == 0:
            continue
        kind = KINDS.get(name, "norm")
        rec = {"max_abs": float(diff.max())}
        if kind == "rel":
            r = diff / ref.clamp_min(1e-300)
            rec.update(max_rel=float(r.max()), rms_rel=float(torch.sqrt((r * r).mean())))
        elif kind == "norm":
            scale = float(ref.max())
            if scale > 0:
                r = diff / scale
                rec.update(max_norm=float(r.max()), rms_norm=float(torch.sqrt((r * r).mean())))
        out[name] = rec
    return out


def drift(d0, d1):
    """Change of mass, momentum and mechanical energy between two diagnostics dicts."""
    e0 = d0["kinetic"] + d0["potential"]
    e1 = d1["kinetic"] + d1["potential"]
    return {"mass_rel": (d1["mass"] - d0["mass"]) / d0["mass"],
            "momentum": [float(x) for x in (d1["momentum"] - d0["momentum"])],
            "energy": e1 - e0, "energy_rel": (e1 - e0) / abs(e0) if e0 else float("nan"),
            "front": d1["front"], "front_advance": d1["front"] - d0["front"]}
