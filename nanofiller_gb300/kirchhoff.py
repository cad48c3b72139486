"""Command-line drop-in for the offline Kirchhoff tool
(tools/kirchhoff/kirchhoff.py) over nf_ac_spectrum:

    python -m nanofiller_gb300.kirchhoff R_cut L_box logF_step [N_patch patch_id]

R_cut: electrostatic range (nm); L_box: box size (um); logF_step: step of the
log10-frequency grid; N_patch / patch_id: the grid split into N_patch patches,
this run doing one (the tool's arguments, kirchhoff.py:34-56). Reads the
tool's four tables from the working directory (segment.La.dat,
internal.DS.dat, source.DS.dat, sink.DS.dat; --coo reads the names the
internal mode writes: segment.LA.coo, internal.DS.coo, source.DS.coo,
sink.DS.coo) and writes kirchhoff.<patch_id>.log and
impedance_rRC.<patch_id>.dat in the tool's formats.

Differences from the tool: the node count is the largest node id in any table
plus one (the tool takes the last segment's J + 1, kirchhoff.py:208); nodes
whose component does not join source and sink are left out of the solve (the
tool keeps them, which leaves its matrix singular when a component floats).
"""
import argparse
import os
import sys

import numpy as np

from . import SNK_ELEC, SRC_ELEC, Simulation, ac_frequencies, configs, write_impedance, write_kirchhoff_log


def read_tables(directory, coo=False):
    names = (("segment.LA.coo", "internal.DS.coo", "source.DS.coo", "sink.DS.coo") if coo else
             ("segment.La.dat", "internal.DS.dat", "source.DS.dat", "sink.DS.dat"))
    paths = [os.path.join(directory, x) for x in names]

    def table(path, cols):
        return np.loadtxt(path, skiprows=1, usecols=cols, ndmin=2).reshape(-1, len(cols))
    sg = table(paths[0], (0, 1, 2, 3))
    it = table(paths[1], (0, 1, 2, 3))
    so = table(paths[2], (1, 2, 3))  # the node is column 1 (kirchhoff.py:136-138)
    si = table(paths[3], (1, 2, 3))
    nodes = np.concatenate([sg[:, 0], sg[:, 1], it[:, 0], it[:, 1], so[:, 0], si[:, 0]])
    return dict(n_nodes=int(nodes.max()) + 1 if len(nodes) else 0,
                seg_i=sg[:, 0].astype(np.uint32), seg_j=sg[:, 1].astype(np.uint32), seg_l=sg[:, 2], seg_a=sg[:, 3],
                ct_i=np.concatenate([it[:, 0], so[:, 0], si[:, 0]]).astype(np.uint32),
                ct_j=np.concatenate([it[:, 1], np.full(len(so), SRC_ELEC), np.full(len(si), SNK_ELEC)]).astype(np.uint32),
                ct_d=np.concatenate([it[:, 2], so[:, 1], si[:, 1]]),
                ct_s=np.concatenate([it[:, 3], so[:, 2], si[:, 2]]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("r_cut", type=float, help="electrostatic range, nm")
    ap.add_argument("l_box", type=float, help="box size, um")
    ap.add_argument("log_df", type=float, help="log10-frequency step")
    ap.add_argument("n_patch", type=int, nargs="?", default=1)
    ap.add_argument("patch_id", type=int, nargs="?", default=0)
    ap.add_argument("--dir", default=".")
    ap.add_argument("--coo", action="store_true", help="read the .coo names of the internal mode")
    ap.add_argument("--sigma", type=float, default=6.7e7, help="rod conductivity, S/m (the tool's s0)")
    a = ap.parse_args(argv)
    net = read_tables(a.dir, a.coo)
    freq = ac_frequencies(a.log_df, a.n_patch, a.patch_id)
    # the handle only supplies a stream, device workspace and rod_sigma; any
    # valid box does
    with Simulation(dict(configs.SMALL, rod_sigma=a.sigma * 1e-6)) as sim:
        spec = sim.ac_spectrum(freq, net=net, check=False, delta_eff=a.r_cut * 1e-3, l_box=a.l_box)
    st = spec["stats"]
    print(f"frequency scale: {st['omega0']}")
    print(f"impedance scale: {st['R0']} {st['C0']}")
    print(f"Number of nodes: {st['n_nodes']}, in the source-sink network: {st['n_active']}")
    elapsed = st["ms"] * 1e-3 / max(len(freq), 1)
    write_kirchhoff_log(os.path.join(a.dir, f"kirchhoff.{a.patch_id}.log"), spec, elapsed)
    write_impedance(os.path.join(a.dir, f"impedance_rRC.{a.patch_id}.dat"), spec)
    bad = int(np.sum(spec["converged"] == 0))
    if bad:
        print(f"{bad} frequencies missed the tolerance", file=sys.stderr)
    return 0 if spec["status"] in (0, 7) else 1


if __name__ == "__main__":
    sys.exit(main())
