"""Scene dictionaries for the benchmark workloads, in the reference's scene-JSON schema.

Every function returns a dict with the ``Configuration`` / ``Materials`` / ``Blocks``
layout that the reference's ``SimConfiger`` reads (README scene-file section).  The
workloads are:

* ``dambreak_2d`` - 2D WCSPH water dambreak: domain 3.22 x 1.6 m, fluid block 1.2 x 0.6 m
  at the origin, spacing 0.01 m, Wendland C2, Tait (rho0 1000, B 5e4, gamma 7),
  viscosity 0.005, leap-frog at dt 1e-4, jitter +-1e-4 m.
* ``dambreak_3d`` - 3D WCSPH dambreak: domain 3.22 x 1.6 x 0.5 m, block 1.2 x 0.6 x 0.2 m,
  spacing 0.0054 m (911,754 fluid + 1,413,114 dummy particles), CSPM correction on, XSPH
  off, leap-frog at dt 2e-5, jitter +-1 % of the spacing.
* ``dambreak_ensemble`` - B independent 2D dambreaks for a batched run: block width
  uniform in [0.3, 1.5] m, height uniform in [0.2, 0.8] m, stiffness log-uniform in
  [2e4, 1e5], viscosity log-uniform in [1e-3, 1e-2], all drawn from one seed (numpy
  PCG64); spacing 0.01 m, leap-frog at dt 1e-4, domain 3.22 x 1.6 m.
* ``column_2d`` - 2D granular column collapse (mu(I) or Drucker-Prager): sand rho0 2040,
  c 0, phi 21.9 deg, E 5.84e6, nu 0.3, psi 0; column 0.2 x 0.1 m at spacing 0.001 m,
  symplectic Euler at dt 1e-5, jitter +-1 % of the spacing.
"""


def _cfg(**kw):
    base = {
        "GPUmemoryPercent": 0.1, "is2D": True,
        "domainStart": [0.0, 0.0, 0.0], "domainEnd": [3.22, 1.6, 0.5],
        "gravitation": [0.0, -9.81, 0.0], "particleRadius": 0.005, "kappa": 2.0, "kh": 1.5,
        "simulationMethod": 1, "timeStepSizeMin": 1e-4, "boundary": 2, "kernel": 1,
        "kernelCorrection": 0, "timeIntegration": 2, "xsph": False,
        # presentation keys of the scene schema (read by the reference's constructors)
        "colorTitle": 2, "colorGroup": 0, "showBdyPts": False, "stepsPerRenderUpdate": 10,
    }
    base.update(kw)
    return base


def water(viscosity=0.005, stiffness=50000.0, density0=1000.0, exponent=7):
    return {"matId": 0, "matType": 1, "color": [50, 100, 200], "density0": density0,
            "viscosity": viscosity, "stiffness": stiffness, "exponent": exponent}


def sand(density0=2040.0, cohesion=0.0, friction=21.9, E=5.84e6, poison=0.3, dilatancy=0.0):
    return {"matId": 0, "matType": 2, "color": [180, 100, 24], "density0": density0,
            "cohesion": cohesion, "friction": friction, "EYoungMod": E, "poison": poison,
            "dilatancy": dilatancy}


def block(size, translation=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0), material=0, obj=0):
    return {"objectId": obj, "size": list(size), "translation": list(translation),
            "velocity": list(velocity), "materialId": material}


def dambreak_2d(spacing=0.01, width=1.2, height=0.6, dt=1e-4, jitter=1e-4, seed=1,
                stiffness=50000.0, viscosity=0.005, integration=2, kernel=1, corr=0, xsph=False,
                domain=(3.22, 1.6)):
    return {
        "Configuration": _cfg(particleRadius=spacing / 2, timeStepSizeMin=dt, jitter=jitter, seed=seed,
                              domainEnd=[domain[0], domain[1], 0.5], timeIntegration=integration,
                              kernel=kernel, kernelCorrection=corr, xsph=xsph),
        "Materials": [water(viscosity=viscosity, stiffness=stiffness)],
        "Blocks": [block((width, height, 0.1))],
    }


def dambreak_3d(spacing=0.0054, dt=2e-5, jitter_frac=0.01, seed=2, corr=1, integration=2,
                domain=(3.22, 1.6, 0.5), size=(1.2, 0.6, 0.2)):
    return {
        "Configuration": _cfg(is2D=False, particleRadius=spacing / 2, timeStepSizeMin=dt,
                              domainEnd=list(domain), kernelCorrection=corr, timeIntegration=integration,
                              jitter=jitter_frac * spacing, seed=seed),
        "Materials": [water()],
        "Blocks": [block(size)],
    }


def column_2d(method=3, spacing=0.001, dt=1e-5, jitter_frac=0.01, seed=3, integration=1,
              width=0.2, height=0.1, domain=(0.5, 0.15), xsph=False, corr=0):
    return {
        "Configuration": _cfg(particleRadius=spacing / 2, timeStepSizeMin=dt, simulationMethod=method,
                              domainEnd=[domain[0], domain[1], 0.05], timeIntegration=integration,
                              jitter=jitter_frac * spacing, seed=seed, xsph=xsph, kernelCorrection=corr),
        "Materials": [sand()],
        "Blocks": [block((width, height, 0.05))],
    }


def floating_box_2d(spacing=0.02, dt=1e-4, jitter=2e-4, seed=5, integration=2, box_density=500.0,
                    box=(0.12, 0.08), box_at=(0.24, 0.4), water=(0.6, 0.4), domain=(1.2, 0.8), xsph=False, corr=0):
    """A 2D water column with a dynamic rigid box resting on its surface: the box (shape
    matching, eng/solver_sph_base.py:467-518) feels the water's pressure and viscous
    reaction and gravity; rigid material type 11, isDynamic true."""
    d = dambreak_2d(spacing=spacing, width=water[0], height=water[1], dt=dt, jitter=jitter, seed=seed,
                    integration=integration, domain=domain, xsph=xsph, corr=corr)
    d["Materials"].append({"matId": 1, "matType": 11, "color": [155, 55, 55], "density0": box_density})
    b = block((box[0], box[1], 0.05), translation=(box_at[0], box_at[1], 0.0), material=1, obj=1)
    b["isDynamic"] = True
    d["Blocks"].append(b)
    return d


def floating_box_3d(spacing=0.02, dt=2e-5, jitter_frac=0.01, seed=6, integration=2, box_density=500.0, corr=1):
    """The 3D counterpart of floating_box_2d: water 0.3 x 0.2 x 0.16 m in a 0.6 x 0.4 x 0.2 m
    domain, a 0.1 x 0.06 x 0.08 m dynamic rigid box on the surface."""
    d = dambreak_3d(spacing=spacing, dt=dt, jitter_frac=jitter_frac, seed=seed, corr=corr, integration=integration,
                    domain=(0.6, 0.4, 0.2), size=(0.3, 0.2, 0.16))
    d["Materials"].append({"matId": 1, "matType": 11, "color": [155, 55, 55], "density0": box_density})
    b = block((0.1, 0.06, 0.08), translation=(0.1, 0.2, 0.04), material=1, obj=1)
    b["isDynamic"] = True
    d["Blocks"].append(b)
    return d


def dambreak_ensemble(n=256, seed=7, spacing=0.01, dt=1e-4, width=(0.3, 1.5), height=(0.2, 0.8),
                      stiffness=(2e4, 1e5), viscosity=(1e-3, 1e-2), domain=(3.22, 1.6), jitter=1e-4):
    """Scene dicts of an ensemble of 2D dambreaks with seeded block sizes and fluid parameters."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for q in range(n):
        w = float(rng.uniform(*width))
        hgt = float(rng.uniform(*height))
        b = float(np.exp(rng.uniform(np.log(stiffness[0]), np.log(stiffness[1]))))
        nu = float(np.exp(rng.uniform(np.log(viscosity[0]), np.log(viscosity[1]))))
        # whole lattice rows / columns, as the reference's generator fills the block
        w = round(w / spacing) * spacing
        hgt = round(hgt / spacing) * spacing
        out.append(dambreak_2d(spacing=spacing, width=w, height=hgt, dt=dt, jitter=jitter, seed=seed * 100003 + q,
                               stiffness=b, viscosity=nu, domain=domain))
    return out
