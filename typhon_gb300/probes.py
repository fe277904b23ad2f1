"""Volume probes of a zone (Typhon's BLOCK:PROBE with TYPE = VOL_MIN | VOL_MAX | VOL_AVERAGE).

Typhon evaluates a probe's QUANTITY, a symbolic expression of the zone's primitive fields,
over the interior cells and reduces it (CFDTOOLS/Mesh/PROBECALC.f90:22-212, called from
SOURCE/ZONE/prb_zone_vol.f90 at the end of each cycle): the minimum, the maximum, or the
volume-weighted average sum(q V) / sum(V).  The names an expression may use are those
prb_vol_calc puts in its function environment: each scalar field by its quantity name (RHO,
PS for a Navier-Stokes zone, TS for heat conduction), each vector field by its name as its
magnitude (V = |velocity|) and by its components (V_X, V_Y, V_Z), the cell centre (x, y, z)
and the time t.  Expressions are parsed here with Python's ast module and evaluated on numpy
arrays: numbers, names, + - * / ** and unary minus, and the functions sqrt, abs, exp, log,
log10, sin, cos, tan, min, max.
"""
import ast

import numpy as np

_FUNCS = {"sqrt": np.sqrt, "abs": np.abs, "exp": np.exp, "log": np.log, "log10": np.log10, "sin": np.sin,
          "cos": np.cos, "tan": np.tan, "min": np.minimum, "max": np.maximum}
_BINOPS = {ast.Add: np.add, ast.Sub: np.subtract, ast.Mult: np.multiply, ast.Div: np.divide, ast.Pow: np.power}


class ProbeError(ValueError):
    pass


def evaluate(expr, env):
    """The value of the expression `expr` (a string) with the names of `env` (case-blind)."""
    names = {k.upper(): v for k, v in env.items()}
    tree = ast.parse(expr.strip(), mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name):
            if n.id.upper() not in names:
                raise ProbeError(f"unknown quantity {n.id} in {expr!r}")
            return names[n.id.upper()]
        if isinstance(n, ast.BinOp) and type(n.op) in _BINOPS:
            return _BINOPS[type(n.op)](ev(n.left), ev(n.right))
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id.lower() in _FUNCS \
                and not n.keywords:
            return _FUNCS[n.func.id.lower()](*[ev(a) for a in n.args])
        raise ProbeError(f"unsupported expression {expr!r}")

    return ev(tree)


def ns_environment(prim, centre=None, time=0.0):
    """Names of a Navier-Stokes zone: prim is (rho, p, u, v, w) per interior cell."""
    q = np.asarray(prim, np.float64)
    env = {"RHO": q[0], "PS": q[1], "V": np.sqrt(q[2] * q[2] + q[3] * q[3] + q[4] * q[4]),
           "V_X": q[2], "V_Y": q[3], "V_Z": q[4], "t": time}
    if centre is not None:
        c = np.asarray(centre, np.float64)
        env.update(x=c[:, 0], y=c[:, 1], z=c[:, 2])
    return env


def vol_probe(kind, expr, env, volume):
    """VOL_MIN, VOL_MAX or VOL_AVERAGE of expr over the cells (volume: their volumes)."""
    q = np.broadcast_to(np.asarray(evaluate(expr, env), np.float64), np.shape(volume))
    kind = kind.upper()
    if kind == "VOL_MIN":
        return float(q.min())
    if kind == "VOL_MAX":
        return float(q.max())
    if kind == "VOL_AVERAGE":
        v = np.asarray(volume, np.float64)
        return float(np.sum(q * v) / np.sum(v))
    raise ProbeError(f"unknown probe type {kind}")
