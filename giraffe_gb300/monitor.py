"""Monitor files in the reference's format (reference src/Monitor.cpp:280-
401, src/Node.cpp:227-320): one text file per monitored node,
monitors/monitor_node_<id>.txt, a header line and one line per monitored
time with Node::WriteMonitor's 31 columns, every value as %.6e.

The lines come from the device run (gpu.BatchSolver.monitor, gf_batch_monitor):
the library keeps them while a structure with a Monitor block runs, so a
served or batched deck can be diffed line by line against the reference's
own monitor files.
"""
from __future__ import annotations

import os

import numpy as np

HEADER = ("TIME\tX\tY\tZ\tROTX\tROTY\tROTZ\tFX\tFY\tFZ\tMX\tMY\tMZ\tFXloc\tFYloc\tFZloc\tMXloc\tMYloc\tMZloc\t"
          "dX\tdY\tdZ\tdROTX\tdROTY\tdROTZ\tddX\tddY\tddZ\tddROTX\tddROTY\tddROTZ")


def node_lines(lines: np.ndarray) -> str:
    """The text of one node's monitor file: the header, then each line's 31
    values as %.6e separated by tabs."""
    out = [HEADER]
    for row in np.asarray(lines):
        out.append("\t".join("%.6e" % v for v in row))
    return "\n".join(out) + "\n"


def write_node_monitors(structure, lines: np.ndarray, folder: str) -> list:
    """Writes monitors/monitor_node_<id>.txt under folder for each of the
    structure's monitored nodes (ids 1-based, as in the deck); lines is
    [node][line][31].  Returns the paths written."""
    if structure.monitor is None or not structure.monitor.nodes:
        return []
    d = os.path.join(folder, "monitors")
    os.makedirs(d, exist_ok=True)
    paths = []
    for q, node in enumerate(structure.monitor.nodes):
        path = os.path.join(d, f"monitor_node_{int(node) + 1}.txt")
        with open(path, "w") as f:
            f.write(node_lines(lines[q]))
        paths.append(path)
    return paths
