"""Case setup for the structured-grid flat-plate workloads.

Writes and reads the same two inputs the reference driver consumes
(src/main.cpp:24-42): a TOML ``.inp`` file with the keys of
src/utils/config.cpp:32-87 plus ``[[boundary]]`` tables (src/model/bc.cpp:465-526),
and a single-block plot3d grid file read by Mesh::plot3d_loader
(src/utils/mesh.cpp:156-169: ``nblock``, ``ni nj``, then all x with i fastest,
then all y).

Non-dimensionalisation follows the reference's fluid model
(src/model/fluid.cpp:12): R = p_inf/(rho_inf*T_inf).  With rho_inf = 1 and
p_inf = T_inf = 1/gamma the freestream sound speed is 1, so u_inf = Mach and
mu_inf = Mach/Re_L for a plate of unit length.

Grid rules (the workload statements leave them open, so they are fixed here):
  * x is uniform on [x_min, x_max]; the plate starts at the vertex nearest x=0
    (x=0 rarely falls on a vertex of a uniform grid).
  * y grows geometrically from the first height h1 at ratio r.  If that
    growth reaches y_max early, the spacing is frozen and the remaining cells
    are uniform up to y_max.  If it cannot reach y_max at all, the ratio is
    raised until nj-1 geometric cells end exactly at y_max.
  * An inclined top boundary scales each column's y distribution so the top
    vertex lies on y_max + (x - x_min) * tan(angle).
"""
from __future__ import annotations

import dataclasses
import math
import os
import tomllib
from typing import Optional

import numpy as np

GAMMA = 1.4


# --------------------------------------------------------------------------
# grids
# --------------------------------------------------------------------------
def stretched_spacing(n_cells: int, h1: float, ratio: float, y_max: float) -> np.ndarray:
    """Vertex y-coordinates (n_cells+1) from the growth rule in the module docstring."""
    def geo_sum(r, m):
        return h1 * m if abs(r - 1.0) < 1e-15 else h1 * (r ** m - 1.0) / (r - 1.0)

    if geo_sum(ratio, n_cells) < y_max:
        lo, hi = ratio, 4.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if geo_sum(mid, n_cells) < y_max:
                lo = mid
            else:
                hi = mid
        r = 0.5 * (lo + hi)
        dy = h1 * r ** np.arange(n_cells)
        y = np.concatenate([[0.0], np.cumsum(dy)])
        y *= y_max / y[-1]
        return y
    m = 0
    while m < n_cells and geo_sum(ratio, m + 1) + (n_cells - m - 1) * h1 * ratio ** (m + 1) <= y_max:
        m += 1
    dy_geo = h1 * ratio ** np.arange(m)
    s = dy_geo.sum()
    rest = n_cells - m
    dy = np.concatenate([dy_geo, np.full(rest, (y_max - s) / rest)]) if rest > 0 else dy_geo
    y = np.concatenate([[0.0], np.cumsum(dy)])
    y[-1] = y_max
    return y


@dataclasses.dataclass
class Grid:
    xv: np.ndarray   # [ni][nj]
    yv: np.ndarray   # [ni][nj]
    i_le: int        # vertex index where the no-slip plate starts

    @property
    def ni(self) -> int:
        return self.xv.shape[0]

    @property
    def nj(self) -> int:
        return self.xv.shape[1]


def flat_plate_grid(ni: int, nj: int, x_min=-0.25, x_max=1.0, y_max=0.5,
                    h1=1e-4, ratio=1.08, top_angle_deg=0.0) -> Grid:
    x = np.linspace(x_min, x_max, ni)
    i_le = int(np.argmin(np.abs(x)))
    y = stretched_spacing(nj - 1, h1, ratio, y_max)
    xv = np.repeat(x[:, None], nj, axis=1)
    top = y_max + (x - x_min) * math.tan(math.radians(top_angle_deg))
    yv = y[None, :] * (top / y_max)[:, None]
    return Grid(np.ascontiguousarray(xv), np.ascontiguousarray(yv), i_le)


def write_p3d(path: str, grid: Grid) -> None:
    """plot3d text format read by src/utils/mesh.cpp:156-169."""
    with open(path, "w") as f:
        f.write("1\n%d %d\n" % (grid.ni, grid.nj))
        np.savetxt(f, grid.xv.T.reshape(-1), fmt="%.20e")
        np.savetxt(f, grid.yv.T.reshape(-1), fmt="%.20e")


def read_p3d(path: str) -> tuple[np.ndarray, np.ndarray]:
    with open(path) as f:
        toks = f.read().split()
    nb, ni, nj = int(toks[0]), int(toks[1]), int(toks[2])
    if nb != 1:
        raise ValueError("only single-block plot3d grids are supported")
    vals = np.array(toks[3:3 + 2 * ni * nj], dtype=np.float64)
    if vals.size != 2 * ni * nj:
        raise ValueError("truncated plot3d grid %s" % path)
    xv = vals[:ni * nj].reshape(nj, ni).T.copy()
    yv = vals[ni * nj:].reshape(nj, ni).T.copy()
    return xv, yv


def read_simple(path: str, ni: int, nj: int) -> tuple[np.ndarray, np.ndarray]:
    """``simple`` format of src/utils/mesh.cpp:134-142: x y pairs, i fastest."""
    vals = np.loadtxt(path, dtype=np.float64).reshape(-1)
    if vals.size < 2 * ni * nj:
        raise ValueError("truncated simple grid %s" % path)
    xy = vals[:2 * ni * nj].reshape(nj, ni, 2)
    return xy[:, :, 0].T.copy(), xy[:, :, 1].T.copy()


# --------------------------------------------------------------------------
# case description
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Boundary:
    type: str     # freestream | slipwall | wall | outflow | periodic | isothermalwall | wake
    face: str     # bottom | right | top | left
    start: int
    end: int      # negative counts from the end of the ghost-padded range
    u: float = 0.0
    v: float = 0.0
    T: float = 0.0


@dataclasses.dataclass
class Case:
    grid_path: str
    ni: int
    nj: int
    rho_inf: float = 1.0
    u_inf: float = 0.0
    v_inf: float = 0.0
    p_inf: float = 1.0 / GAMMA
    T_inf: float = 1.0 / GAMMA
    mu_inf: float = 0.0
    pr_inf: float = 0.7
    aoa: float = 0.0
    order: int = 2
    lhs_order: Optional[int] = None
    flux: str = "roe"
    scheme: str = "forward_euler"
    cfl: float = 1.0
    cfl_ramp: bool = False
    cfl_ramp_iteration: int = 20
    cfl_ramp_exponent: float = 1.1
    under_relaxation: float = 1.0
    under_relaxation_ramp: bool = False
    under_relaxation_ramp_iteration: int = 20
    under_relaxation_ramp_exponent: float = 1.1
    tolerance: float = 1e10
    iteration_max: int = 1
    dpdx: float = 0.0
    dpdy: float = 0.0
    label: str = "flow"
    tail: int = 0
    grid_format: str = "p3d"
    boundaries: list = dataclasses.field(default_factory=list)
    # keys this project adds (the reference ignores unknown keys)
    viscosity_law: str = "power"        # power (reference, fluid.cpp:38-40) | sutherland
    turbulence: str = "none"            # none | sa
    nu_tilde_inf_ratio: float = 3.0     # nu_tilde_inf / nu_inf
    i_le: int = -1                      # plate start vertex (drag integral bounds)
    plate_x_end: float = 1.0

    @property
    def nq(self) -> int:
        return 5 if self.turbulence == "sa" else 4

    @property
    def nic(self) -> int:
        return self.ni - 1

    @property
    def njc(self) -> int:
        return self.nj - 1


def _toml_value(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return repr(float(v))
    return '"%s"' % v


def write_inp(path: str, c: Case) -> None:
    """Writes the reference's TOML keys (src/utils/config.cpp:32-87)."""
    lines = ["[geometry]",
             "filename = %s" % _toml_value(c.grid_path),
             "ni = %d" % c.ni, "nj = %d" % c.nj, "tail = %d" % c.tail,
             "format = %s" % _toml_value(c.grid_format), "",
             "[freestream]"]
    for k in ("rho_inf", "u_inf", "v_inf", "p_inf", "T_inf", "mu_inf", "pr_inf", "aoa"):
        lines.append("%s = %s" % (k, _toml_value(float(getattr(c, k)))))
    lines.append("viscosity_law = %s" % _toml_value(c.viscosity_law))
    lines += ["", "[source]", "dpdx = %s" % _toml_value(float(c.dpdx)),
              "dpdy = %s" % _toml_value(float(c.dpdy)), "", "[solver]"]
    lines.append("order = %d" % c.order)
    lines.append("lhs_order = %d" % (c.lhs_order if c.lhs_order is not None else c.order))
    for k in ("flux", "scheme"):
        lines.append("%s = %s" % (k, _toml_value(getattr(c, k))))
    for k in ("cfl", "cfl_ramp", "cfl_ramp_iteration", "cfl_ramp_exponent",
              "under_relaxation", "under_relaxation_ramp", "under_relaxation_ramp_iteration",
              "under_relaxation_ramp_exponent", "tolerance", "iteration_max"):
        lines.append("%s = %s" % (k, _toml_value(getattr(c, k))))
    lines += ["", "[turbulence]", "model = %s" % _toml_value(c.turbulence),
              "nu_tilde_inf_ratio = %s" % _toml_value(float(c.nu_tilde_inf_ratio)),
              "", "[objective]", "plate_vertex = %d" % c.i_le,
              "x_end = %s" % _toml_value(float(c.plate_x_end)),
              "", "[io]", "label = %s" % _toml_value(c.label), "restart = false",
              "stdout_frequency = 1", "fileout_frequency = 1000000000", ""]
    for b in c.boundaries:
        lines += ["[[boundary]]", 'name = ""', "type = %s" % _toml_value(b.type),
                  "face = %s" % _toml_value(b.face), "start = %d" % b.start, "end = %d" % b.end]
        if b.type in ("wall", "isothermalwall"):
            lines += ["u = %s" % repr(float(b.u)), "v = %s" % repr(float(b.v))]
        if b.type == "isothermalwall":
            lines.append("T = %s" % repr(float(b.T)))
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines))


def read_inp(path: str) -> Case:
    """Reads a reference ``.inp``; defaults follow src/utils/config.cpp:32-87."""
    with open(path, "rb") as f:
        t = tomllib.load(f)
    g = t.get("geometry", {})
    fs = t.get("freestream", {})
    so = t.get("solver", {})
    src = t.get("source", {})
    io = t.get("io", {})
    tu = t.get("turbulence", {})
    ob = t.get("objective", {})
    grid_path = g.get("filename", "grid.unf2")
    if not os.path.isabs(grid_path):
        grid_path = os.path.join(os.path.dirname(os.path.abspath(path)), grid_path)
    order = int(so.get("order", 1))
    c = Case(grid_path=grid_path, ni=int(g.get("ni", 0)), nj=int(g.get("nj", 0)),
             rho_inf=float(fs.get("rho_inf", 1.0)), u_inf=float(fs.get("u_inf", 0.0)),
             v_inf=float(fs.get("v_inf", 0.0)), p_inf=float(fs.get("p_inf", 1.0 / 1.4)),
             T_inf=float(fs.get("T_inf", 1.0 / 1.4)), mu_inf=float(fs.get("mu_inf", 0.0)),
             pr_inf=float(fs.get("pr_inf", 0.7)),
             aoa=float(fs.get("aoa", 0.0)),
             order=order, lhs_order=int(so.get("lhs_order", order)),
             flux=so.get("flux", "ausm"), scheme=so.get("scheme", "forward_euler"),
             cfl=float(so.get("cfl", 1.0)), cfl_ramp=bool(so.get("cfl_ramp", False)),
             cfl_ramp_iteration=int(so.get("cfl_ramp_iteration", 20)),
             cfl_ramp_exponent=float(so.get("cfl_ramp_exponent", 1.1)),
             under_relaxation=float(so.get("under_relaxation", 1.0)),
             under_relaxation_ramp=bool(so.get("under_relaxation_ramp", False)),
             under_relaxation_ramp_iteration=int(so.get("under_relaxation_ramp_iteration", 20)),
             under_relaxation_ramp_exponent=float(so.get("under_relaxation_ramp_exponent", 1.1)),
             tolerance=float(so.get("tolerance", 1e10)),
             iteration_max=int(so.get("iteration_max", 1)),
             dpdx=float(src.get("dpdx", 0.0)), dpdy=float(src.get("dpdy", 0.0)),
             label=io.get("label", "flow"), tail=int(g.get("tail", 0)),
             grid_format=g.get("format", "grid.unf2"),
             viscosity_law=fs.get("viscosity_law", "power"),
             turbulence=tu.get("model", "none"),
             nu_tilde_inf_ratio=float(tu.get("nu_tilde_inf_ratio", 3.0)),
             i_le=int(ob.get("plate_vertex", -1)), plate_x_end=float(ob.get("x_end", 1.0)))
    for b in t.get("boundary", []):
        c.boundaries.append(Boundary(type=b.get("type", ""), face=b.get("face", ""),
                                     start=int(b.get("start", 0)), end=int(b.get("end", 0)),
                                     u=float(b.get("u", 0.0)), v=float(b.get("v", 0.0)),
                                     T=float(b.get("T", 0.0))))
    return c


def load_grid(c: Case) -> tuple[np.ndarray, np.ndarray]:
    if c.grid_format == "p3d":
        return read_p3d(c.grid_path)
    if c.grid_format == "simple":
        return read_simple(c.grid_path, c.ni, c.nj)
    raise ValueError("unknown grid format %r" % c.grid_format)


def flat_plate_boundaries(i_le: int, top: str = "freestream") -> list:
    """Flat-plate ghost-cell boundary list, in application order.

    Indices are ghost-padded (0..nic+1 along a bottom/top face).  Ghost column
    i covers physical cell i-1; cells left of vertex i_le form the symmetry
    plane, cells from i_le on the no-slip plate.  The order fixes every corner
    ghost: the bottom BCs stop at nic (end=-2), the top and left BCs cover
    their whole ghost row, and the outflow BC runs last so it copies the
    bottom and top ghosts into the right-hand corners (the reference's outflow
    copies its inner neighbour, src/model/bc.cpp:301-307).
    """
    return [Boundary("slipwall", "bottom", 1, i_le),
            Boundary("wall", "bottom", i_le + 1, -2),
            Boundary(top, "top", 0 if top == "freestream" else 1, -1 if top == "freestream" else -2),
            Boundary("freestream", "left", 0, -1),
            Boundary("outflow", "right", 0, -1)]


def flat_plate_case(workdir: str, name: str, ni: int, nj: int, mach: float, reynolds: float,
                    h1: float, ratio: float, y_max: float = 0.5, x_min: float = -0.25,
                    x_max: float = 1.0, top_angle_deg: float = 0.0, turbulence: str = "none",
                    pr: float = 0.72, viscosity_law: str = "power", write_files: bool = True,
                    **solver) -> Case:
    """Writes grid + ``.inp`` for one flat-plate workload and returns the Case.
    With write_files=False nothing is written; the grid is then regenerated
    by flat_plate_grid() with the same arguments."""
    grid = flat_plate_grid(ni, nj, x_min, x_max, y_max, h1, ratio, top_angle_deg)
    grid_path = os.path.join(workdir, name + ".p3d")
    if write_files:
        os.makedirs(workdir, exist_ok=True)
        write_p3d(grid_path, grid)
    top = "freestream" if abs(top_angle_deg) < 1e-12 else "slipwall"
    c = Case(grid_path=grid_path, ni=ni, nj=nj, u_inf=float(mach), mu_inf=float(mach / reynolds),
             pr_inf=pr, flux="roe", boundaries=flat_plate_boundaries(grid.i_le, top),
             turbulence=turbulence, viscosity_law=viscosity_law, i_le=grid.i_le,
             label=os.path.join(workdir, name))
    for k, v in solver.items():
        setattr(c, k, v)
    if write_files:
        write_inp(os.path.join(workdir, name + ".inp"), c)
    return c


# --------------------------------------------------------------------------
# states
# --------------------------------------------------------------------------
def conserved_from_primitive(rho, u, v, p, nut=None) -> np.ndarray:
    """Q = (rho, rho u, rho v, rho E[, rho nu_tilde]) per cell, reference layout
    q[i][j][k] (src/solver/solution.cpp:28, src/model/eulerequation.cpp:262-276)."""
    rhoE = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v)
    comps = [rho, rho * u, rho * v, rhoE]
    if nut is not None:
        comps.append(rho * nut)
    return np.ascontiguousarray(np.stack(comps, axis=-1))


def freestream_state(c: Case) -> np.ndarray:
    shape = (c.nic, c.njc)
    one = np.ones(shape)
    nut = None
    if c.turbulence == "sa":
        nut = one * c.nu_tilde_inf_ratio * c.mu_inf / c.rho_inf
    return conserved_from_primitive(one * c.rho_inf, one * c.u_inf, one * c.v_inf, one * c.p_inf, nut)


def perturbed_state(c: Case, seed: int, amplitude: float = 0.01) -> np.ndarray:
    """Freestream with i.i.d. Gaussian perturbations of relative size
    ``amplitude`` on rho, u, p and nu_tilde and absolute size amplitude*u_inf
    on v; numpy PCG64 stream from ``seed``."""
    rng = np.random.default_rng(seed)
    shape = (c.nic, c.njc)
    rho = c.rho_inf * (1.0 + amplitude * rng.standard_normal(shape))
    u = c.u_inf * (1.0 + amplitude * rng.standard_normal(shape))
    v = c.v_inf + amplitude * c.u_inf * rng.standard_normal(shape)
    p = c.p_inf * (1.0 + amplitude * rng.standard_normal(shape))
    nut = None
    if c.turbulence == "sa":
        base = c.nu_tilde_inf_ratio * c.mu_inf / c.rho_inf
        nut = base * (1.0 + amplitude * rng.standard_normal(shape))
    return conserved_from_primitive(rho, u, v, p, nut)


def case_to_dict(c: Case) -> dict:
    d = dataclasses.asdict(c)
    return d


def case_from_dict(d: dict) -> Case:
    d = dict(d)
    bcs = [Boundary(**b) for b in d.pop("boundaries", [])]
    c = Case(**d)
    c.boundaries = bcs
    return c


def channel_case(workdir: str, name: str, nj: int = 101, height: float = 0.1, ni: int = 3,
                 dx: float = 1e-3, mu: float = 1e-2, dpdx: float = -0.02592, order: int = 2) -> Case:
    """Pressure-driven channel with periodic inflow/outflow and isothermal walls,
    the setup of the reference's examples/laminar/channel/*.inp (3x101 grid,
    h = 0.1, mu = 1e-2, dp/dx = -0.02592)."""
    os.makedirs(workdir, exist_ok=True)
    x = np.arange(ni) * dx
    y = np.linspace(0.0, height, nj)
    xv = np.ascontiguousarray(np.repeat(x[:, None], nj, axis=1))
    yv = np.ascontiguousarray(np.repeat(y[None, :], ni, axis=0))
    grid_path = os.path.join(workdir, name + ".p3d")
    write_p3d(grid_path, Grid(xv, yv, 0))
    T_wall = 1.0 / GAMMA
    c = Case(grid_path=grid_path, ni=ni, nj=nj, u_inf=0.01, mu_inf=mu, pr_inf=0.7, dpdx=dpdx,
             order=order, flux="roe", label=os.path.join(workdir, name),
             boundaries=[Boundary("isothermalwall", "top", 1, -2, 0.0, 0.0, T_wall),
                         Boundary("isothermalwall", "bottom", 1, -2, 0.0, 0.0, T_wall),
                         Boundary("periodic", "left", 0, -1)])
    write_inp(os.path.join(workdir, name + ".inp"), c)
    return c


# --------------------------------------------------------------------------
# C-grid around a NACA 0012 (the reference's examples/laminar/naca0012 setup)
# --------------------------------------------------------------------------
def naca0012_half_thickness(x: np.ndarray) -> np.ndarray:
    """NACA four-digit thickness distribution for t = 0.12 with the closed
    trailing edge variant (x^4 coefficient -0.1036)."""
    return 0.6 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)


def naca0012_cgrid(ni: int = 281, nj: int = 151, tail: int = 41, radius: float = 5.0, x_far: float = 6.0,
                   h1: float = 1e-3, ratio: float = 1.1) -> Grid:
    """C-grid by transfinite interpolation between the inner curve (lower wake
    from x_far to the trailing edge, the section clockwise from the lower
    trailing edge round the leading edge, upper wake back to x_far; vertices
    0..tail-1 and ni-tail..ni-1 are the wake, which coincide pairwise) and an
    outer C (a semicircle of `radius` about mid-chord joined to straight lines
    out to x_far).  Inner and outer points correspond by the same parameter
    per segment (x along the wakes, arc length round the section); j is
    stretched from a first spacing of about h1."""
    nbp = ni - 2 * tail + 1  # section panels (the reference's nb, mesh.cpp:349-350)
    if nbp < 4 or nbp % 2:
        raise ValueError("ni - 2 tail + 1 must be even and >= 4")
    half = nbp // 2
    theta = np.linspace(0.0, np.pi, half + 1)
    xl = 0.5 * (1.0 + np.cos(theta))                      # 1 -> 0 (lower)
    xs = np.concatenate([xl, xl[::-1][1:]])                # 1 -> 0 -> 1
    ys = np.concatenate([-naca0012_half_thickness(xl), naca0012_half_thickness(xl[::-1][1:])])
    ys[0] = ys[-1] = 0.0
    dx_te = xs[0] - xs[1]
    wake = 1.0 + stretched_spacing(tail - 1, dx_te, 1.05, x_far - 1.0)  # 1 -> x_far
    xin = np.concatenate([wake[::-1], xs[1:-1], wake])
    yin = np.concatenate([np.zeros(tail), ys[1:-1], np.zeros(tail)])
    assert xin.size == ni
    c0 = 0.5
    xo = np.empty(ni)
    yo = np.empty(ni)
    wf = (wake - 1.0) / (x_far - 1.0)                      # 0 at the trailing edge
    xo[:tail] = (c0 + wf * (x_far - c0))[::-1]
    yo[:tail] = -radius
    xo[ni - tail:] = c0 + wf * (x_far - c0)
    yo[ni - tail:] = radius
    seg = np.hypot(np.diff(xs), np.diff(ys))
    f = np.concatenate([[0.0], np.cumsum(seg)]) / seg.sum()
    phi = -0.5 * np.pi - np.pi * f
    xo[tail - 1:ni - tail + 1] = c0 + radius * np.cos(phi)
    yo[tail - 1:ni - tail + 1] = radius * np.sin(phi)
    s = stretched_spacing(nj - 1, h1 / radius, ratio, 1.0)
    xv = np.ascontiguousarray((1.0 - s)[None, :] * xin[:, None] + s[None, :] * xo[:, None])
    yv = np.ascontiguousarray((1.0 - s)[None, :] * yin[:, None] + s[None, :] * yo[:, None])
    return Grid(xv, yv, tail - 1)


def naca0012_case(workdir: str, name: str, ni: int = 281, nj: int = 151, tail: int = 41, mach: float = 0.5,
                  aoa_deg: float = 1.0, mu: float = 1e-4, write_files: bool = True, **grid) -> Case:
    """The laminar NACA 0012 example's flow and boundaries (freestream on the
    outer C and both outflow ends, wake cut on bottom cells 1..tail-1, no-slip
    wall on the section) on the generated C-grid."""
    g = naca0012_cgrid(ni, nj, tail, **grid)
    grid_path = os.path.join(workdir, name + ".p3d")
    a = math.radians(aoa_deg)
    c = Case(grid_path=grid_path, ni=ni, nj=nj, u_inf=mach * math.cos(a), v_inf=mach * math.sin(a), mu_inf=mu,
             pr_inf=0.7, aoa=aoa_deg, order=2, lhs_order=1, flux="roe", scheme="rk4_jameson", tail=tail,
             label=os.path.join(workdir, name),
             boundaries=[Boundary("freestream", "top", 0, -1), Boundary("freestream", "left", 0, -1),
                         Boundary("freestream", "right", 0, -1), Boundary("wake", "bottom", 1, tail - 1),
                         Boundary("wall", "bottom", tail, ni - tail)])
    if write_files:
        os.makedirs(workdir, exist_ok=True)
        write_p3d(grid_path, g)
        write_inp(os.path.join(workdir, name + ".inp"), c)
    return c
