"""Problem defaults and strict TOML input decks (drop-in for jathenax/input.py:1-63).

Precedence is problem defaults < deck < command line. Unknown sections, keys
or value types raise ValueError, as in the reference.
"""

import tomllib

# name -> (nx, ny, tlim, output file)  (input.py:6-10)
PROBLEMS = {
    "smooth": (64, 48, 0.2, "periodic_isothermal.npz"),
    "kh": (128, 128, 3.0, "kelvin_helmholtz.npz"),
    "turbulence": (256, 256, 45.0, "driven_seed1618.npz"),
}


def default_settings(name):
    """The defaults of one problem (input.py:21-42)."""
    nx, ny, tlim, filename = PROBLEMS[name]
    driven = name == "turbulence"
    settings = {
        "problem": {"name": name},
        "mesh": {"nx": nx, "ny": ny},
        "time": {"tlim": tlim, "nlim": 100_000, "integrator": "rk3", "cfl_number": 0.4},
        "hydro": {
            "reconstruct": "ppm4", "rsolver": "roe", "iso_sound_speed": 1.0,
            "dfloor": 1.17549e-38 if driven else 1e-10,
            "viscosity": 1.5e-6 if driven else 0.0, "smagorinsky_cs": 0.0,
        },
        "hydro_srcterms": {"drag_rate": 0.3333335 if driven else 0.0},
        "sgs": {"model": "", "weights": ""},
        "output": {"file": filename},
    }
    if driven:
        settings["turb_driving"] = {
            "rseed": 1618, "tcorr": 0.75, "dt_update": 0.0075, "tdriv_start": 0.0,
            "dedt": 0.03703705, "nlow": 3, "nhigh": 5, "npeak": 4.0, "sol_fraction": 1.0,
            "min_kx": -5, "max_kx": 5, "min_ky": -5, "max_ky": 5,
        }
    return settings


def read_input(path, problem=None):
    """Load a deck over the selected problem's defaults (input.py:13-63)."""
    deck = {}
    if path is not None:
        with open(path, "rb") as handle:
            deck = tomllib.load(handle)
    section = deck.get("problem", {})
    if not isinstance(section, dict):
        raise ValueError("[problem] must be a table")
    name = problem if problem is not None else section.get("name", "smooth")
    if not isinstance(name, str) or name not in PROBLEMS:
        raise ValueError("problem.name must be smooth, kh, or turbulence")
    settings = default_settings(name)
    for table_name, table in deck.items():
        if table_name not in settings:
            raise ValueError(f"unsupported input section [{table_name}] for {name}")
        if not isinstance(table, dict):
            raise ValueError(f"[{table_name}] must be a table")
        target = settings[table_name]
        for key, value in table.items():
            if key not in target:
                raise ValueError(f"unknown input setting {table_name}.{key}")
            expected = type(target[key])
            allowed = (int, float) if expected is float else (expected,)
            if type(value) not in allowed:
                raise ValueError(f"{table_name}.{key} expects {expected.__name__}")
            target[key] = value
    settings["problem"]["name"] = name
    return settings
