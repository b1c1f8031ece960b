"""Shared test systems: the argon case and the reduced-unit LJ liquid, built by the product's
own lattice / velocity generators and mirrored into the oracle."""
import numpy as np

from pis_gb300.lattice import fcc_lattice, fcc_lattice_constant, maxwell_boltzmann, reduced_temperature

KB = 0.0083144621


def argon(nc=10, a=5.26, eps=0.0104, sigma=3.405, rc=None, temperature=100.0, seed=7):
    """4 nc^3 argon atoms on an FCC lattice (a=5.26 A), LJ eps=0.0104, sigma=3.405, rc=2.5 sigma,
    Maxwell-Boltzmann velocities at 100 K (mass 39.948)."""
    rc = 2.5 * sigma if rc is None else rc
    pos = fcc_lattice(a, nc, nc, nc)
    n = len(pos)
    masses = np.array([39.948])
    vel = maxwell_boltzmann(np.full(n, 39.948), temperature, seed)
    return dict(pos=pos, vel=vel, types=np.ones(n, np.int32), masses=masses, h=np.eye(3) * (a * nc),
                table={(1, 1): (eps, sigma, rc)})


def liquid(nc=6, rho=0.8442, t_star=0.72, seed=3):
    a = fcc_lattice_constant(rho)
    pos = fcc_lattice(a, nc, nc, nc)
    n = len(pos)
    vel = maxwell_boltzmann(np.ones(n), reduced_temperature(t_star), seed)
    return dict(pos=pos, vel=vel, types=np.ones(n, np.int32), masses=np.array([1.0]), h=np.eye(3) * (a * nc),
                table={(1, 1): (1.0, 1.0, 2.5)})


def to_oracle(sysd):
    import oracle
    return oracle.System(sysd["pos"], sysd["types"], sysd["masses"], sysd["h"], sysd["table"], velocities=sysd["vel"])


def to_gpu(sysd, precision="fp64", skin=0.3, list_kind="default", fp64_fast=False, mixed_kahan=False, lanes=0,
           batch=0, tma=False, cluster=0, scan=0, tiles=False, plain_graphs=False,
           unfused=False, ref_order=False, list_capacity=0, auto_grow=True, wait_limit=None):
    from pis_gb300.potentials import GpuContext
    ctx = GpuContext(sysd["table"], len(sysd["masses"]), skin=skin, precision=precision, list_kind=list_kind,
                     fp64_fast=fp64_fast, mixed_kahan=mixed_kahan, lanes=lanes, batch=batch, tma=tma,
                     cluster=cluster, scan=scan, tiles=tiles, plain_graphs=plain_graphs,
                     unfused=unfused, ref_order=ref_order, list_capacity=list_capacity, auto_grow=auto_grow,
                     wait_limit=wait_limit)
    ctx.set_state(sysd["pos"], sysd["types"], sysd["masses"], sysd["h"], velocities=sysd["vel"])
    return ctx


def melted(sysd, steps, dt, seed_perturb=None):
    """Advance the state with the oracle (serial reference manager) to get a disordered configuration."""
    o = to_oracle(sysd)
    o.run_nve(dt, steps)
    out = dict(sysd)
    out["pos"], out["vel"] = o.pos.copy(), o.vel.copy()
    return out
