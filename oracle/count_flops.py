"""Count the oracle's algorithmic floating-point operations per cell and RK stage.

TEST INFRASTRUCTURE: the roofline's algorithmic flop count is defined as the
number of arithmetic ufunc evaluations the reference algorithm performs
(add, subtract, multiply, divide, sqrt, min/max/fmin/fmax, abs, copysign,
negative, square; comparisons and selects count zero), summed over all
elements and divided by cells x stages. Run as a script it writes the table
used by bench.py to jathenax_gb300/flops.json:

    python -m oracle.count_flops
"""

import json
from pathlib import Path

import numpy as np

from . import hydro_oracle as H

ARITHMETIC = {np.add, np.subtract, np.multiply, np.true_divide, np.divide, np.sqrt, np.minimum,
              np.maximum, np.fmin, np.fmax, np.absolute, np.copysign, np.negative, np.square,
              np.power, np.floor_divide}


class _Tally:
    count = 0


class Counted(np.ndarray):
    """ndarray whose arithmetic ufunc calls add their output size to _Tally."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        plain = [x.view(np.ndarray) if isinstance(x, Counted) else x for x in inputs]
        if "out" in kwargs:
            kwargs["out"] = tuple(o.view(np.ndarray) if isinstance(o, Counted) else o for o in kwargs["out"])
        result = getattr(ufunc, method)(*plain, **kwargs)
        if ufunc in ARITHMETIC and method == "__call__":
            _Tally.count += int(np.size(result))
        if isinstance(result, np.ndarray):
            return result.view(Counted)
        return result


class _CountingNumpy:
    """Module proxy: array-producing helpers return Counted arrays."""

    def __getattr__(self, name):
        attr = getattr(np, name)
        if isinstance(attr, np.ufunc) or not callable(attr) or isinstance(attr, type):
            return attr

        def call(*args, **kwargs):
            out = attr(*args, **kwargs)
            if isinstance(out, np.ndarray) and not isinstance(out, Counted):
                return out.view(Counted)
            if isinstance(out, tuple):
                return tuple(o.view(Counted) if isinstance(o, np.ndarray) else o for o in out)
            return out
        return call


def flops_per_cell_stage(recon, solver, nvar=4, integrator="rk3", viscous=False, smag=False,
                         drag=False, n=16):
    """Algorithmic flops per cell per RK stage of one isothermal step."""
    rng = np.random.default_rng(0)
    U = np.empty((n, n, nvar))
    U[..., 0] = 1.0 + 0.2 * rng.random((n, n))
    U[..., 1:] = 0.1 * rng.standard_normal((n, n, nvar - 1))
    saved = H.np
    H.np = _CountingNumpy()
    try:
        _Tally.count = 0
        H.step(U.view(Counted), 0.001, 1 / n, 1 / n, 1.0, 1e-10, integrator,
               nu=1e-3 if viscous else 0.0, cs_smag=0.2 if smag else 0.0, drag=0.3 if drag else 0.0,
               recon=recon, solver=solver)
        total = _Tally.count
    finally:
        H.np = saved
    return total / (n * n * len(H.RK_TABLE[integrator]))


def table():
    out = {}
    for nvar in (3, 4):
        for rec in H.RECON:
            for rs in H.RIEMANN:
                out[f"{rec}/{rs}/nvar{nvar}"] = flops_per_cell_stage(rec, rs, nvar)
        out[f"ppm4/roe/nvar{nvar}/viscous"] = flops_per_cell_stage("ppm4", "roe", nvar, viscous=True)
        out[f"ppm4/roe/nvar{nvar}/smagorinsky"] = flops_per_cell_stage("ppm4", "roe", nvar, viscous=True,
                                                                       smag=True)
        out[f"ppm4/roe/nvar{nvar}/viscous_drag"] = flops_per_cell_stage("ppm4", "roe", nvar, viscous=True,
                                                                        drag=True)
    return out


if __name__ == "__main__":
    path = Path(__file__).resolve().parents[1] / "jathenax_gb300" / "flops.json"
    data = {"definition": "arithmetic ufunc evaluations per cell per RK stage of the float64 "
                          "oracle (rk3 step on a 16x16 grid); comparisons/selects count 0",
            "generator": "python -m oracle.count_flops", "flops_per_cell_stage": table()}
    path.write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
    print(path)
    for key, value in data["flops_per_cell_stage"].items():
        print(f"{key:32s} {value:8.2f}")
