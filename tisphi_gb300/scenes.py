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
