"""Throughput of the local-inertial land grid with its river (include/wflow_gb300_li.h).

    python -m wflow_gb300.li_bench [--nx 2048] [--ny 2048] [--substeps 200] [--steps 2]

A synthetic square grid (100 m cells, elevation falling east and toward the river rows) with a
river along every 64th row draining east into one ghost cell per row, from a warm state with
runoff on every cell. Prints one JSON line per measurement: explicit sub-steps at a fixed dt
(the three kernels of a sub-step and the host's wait for them) and whole model steps of one
hour (with the stable-time-step reduction and its read-back before every sub-step), as
cell-substeps/s of land cells, with the algorithmic bytes per land-cell sub-step of the kernels
(land fluxes 224 B, land depths 96 B, the river edges and time step besides) for a roofline.
"""

import argparse
import json
import time

import numpy as np

from .li_river import LiDomain

BYTES_PER_CELL_SUBSTEP = 224 + 96  # li_land_flux_kernel + li_land_depth_kernel, per land cell


def grid(nx, ny, seed=1, river_every=64, cell=100.0):
    rng = np.random.default_rng(seed)
    n = nx * ny
    idx = np.arange(n)
    row, col = np.divmod(idx, nx)
    land = dict(ind_x_up=np.where(col > 0, idx - 1, n), ind_x_down=np.where(col < nx - 1, idx + 1, n),
                ind_y_up=np.where(row > 0, idx - nx, n), ind_y_down=np.where(row < ny - 1, idx + nx, n),
                x_length=np.full(n, cell), y_length=np.full(n, cell))
    rows = np.arange(river_every // 2, ny, river_every)
    r = (row - river_every // 2) % river_every
    dist = np.minimum(r, river_every - r)  # rows to the nearest river row
    land["elevation"] = 0.001 * (nx - col) * cell + 0.002 * dist * cell + rng.uniform(0.0, 0.05, n)
    land["mannings_n_sq"] = rng.uniform(0.03, 0.08, n) ** 2
    cells = (rows[:, None] * nx + np.arange(nx)[None, :]).ravel()  # river cells, row by row
    nra, nrow = len(cells), len(rows)
    river_index = np.full(n, -1, np.int64)
    river_index[cells] = np.arange(nra)
    land["river_index"] = river_index
    width = rng.uniform(10.0, 40.0, nra + nrow)
    land["xwidth_at_edge"] = land["x_length"].copy()
    land["ywidth_at_edge"] = land["y_length"].copy()
    land["ywidth_at_edge"][cells] = np.maximum(cell - width[:nra], 0.0)
    land.update(theta=0.8, h_thresh=1e-3, alpha=0.7, froude_limit=True)
    k = np.arange(nra)
    last = (k % nx) == nx - 1
    src = k.astype(np.int64)
    dst = np.where(last, nra + k // nx, k + 1).astype(np.int64)
    bankfull = rng.uniform(1.0, 2.0, nra + nrow)
    zb = np.concatenate([land["elevation"][cells], land["elevation"][cells[last]] - 0.5]) - bankfull
    fl = np.full(nra + nrow, cell)
    n_manning = rng.uniform(0.025, 0.04, nra + nrow)
    n_e = (n_manning[dst] * fl[dst] + n_manning[src] * fl[src]) / (fl[dst] + fl[src])
    river = dict(n_active=nra, src=src, dst=dst, zb=zb, flow_length=fl, flow_width=width, bankfull_depth=bankfull,
                 zb_edge=np.maximum(zb[src], zb[dst]), width_edge=np.minimum(width[dst], width[src]),
                 length_edge=0.5 * (fl[dst] + fl[src]), mannings_n_sq_edge=n_e * n_e, h_thresh=1e-3, alpha=0.7,
                 froude_limit=True)
    h_river = np.concatenate([rng.uniform(0.3, 1.5, nra), np.full(nrow, 1.0)])
    h_land = rng.uniform(0.0, 0.1, n) * (rng.random(n) < 0.5)
    h_land[cells] = 0.0
    runoff = np.full(n, 5e-3 / 3600.0 * cell * cell)  # 5 mm/h over every cell [m3 s-1]
    return land, river, h_river, h_land, runoff


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=2048)
    ap.add_argument("--substeps", type=int, default=200)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args(argv)
    land, river, h_river, h_land, runoff = grid(a.nx, a.ny)
    n = len(h_land)
    d = LiDomain(land, river, h_river)
    d.set_state(h_land, h_river)
    d.set_inputs(runoff)
    dt_s = d.stable_timestep()
    for _ in range(a.warmup):
        d.substep(dt_s)
    t0 = time.perf_counter()
    for _ in range(a.substeps):
        d.substep(dt_s)
    t_sub = (time.perf_counter() - t0) / a.substeps
    base = dict(unit="cell-substeps/s", n_land=n, n_river=int(river["n_active"]), dtype="f64",
                bytes_per_cell_substep=BYTES_PER_CELL_SUBSTEP)
    print(json.dumps(dict(base, metric="li_domain_substep", value=n / t_sub, ms_per_substep=t_sub * 1e3,
                          achieved_gbs=n * BYTES_PER_CELL_SUBSTEP / t_sub / 1e9)))
    t0 = time.perf_counter()
    k = sum(d.step(3600.0) for _ in range(a.steps))
    t_step = time.perf_counter() - t0
    print(json.dumps(dict(base, metric="li_domain_model_step", value=n * k / t_step, substeps=k,
                          ms_per_step=t_step / a.steps * 1e3)))
    d.close()


if __name__ == "__main__":
    main()
