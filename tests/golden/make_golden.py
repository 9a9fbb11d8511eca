"""Regenerates the golden fixtures of the reference's 2d_hilltop case and its
1-D example mesh.

Reads, from a checkout of the reference (the path given as the only
argument):
  residuals.csv                          per-step residual trace of a reference run
  cases/2d_hilltop/2d_hilltop_fs.msh     its mesh
  cases/2d_hilltop/2d_hilltop.json       its configuration
  doc/1d/line.msh                        the 1-D example mesh (100 lines on [-5, 5])
and writes next to this script:
  hilltop_residuals.csv   time;res_p;res_rho;res_vx;res_vy (elapsed time dropped)
  2d_hilltop_fs.msh.gz    the mesh, gzip-compressed
  2d_hilltop.json         the configuration with the mesh path made relative
  line_1d.msh             the 1-D mesh as is
"""
import gzip
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    rows = open(os.path.join(ref, "residuals.csv")).read().strip().splitlines()
    with open(os.path.join(HERE, "hilltop_residuals.csv"), "w") as f:
        f.write("time;res_p;res_rho;res_vx;res_vy\n")
        for r in rows[1:]:
            c = r.split(";")
            f.write(";".join(c[:5]) + "\n")
    with open(os.path.join(ref, "cases/2d_hilltop/2d_hilltop_fs.msh"), "rb") as src:
        data = src.read()
    with gzip.GzipFile(os.path.join(HERE, "2d_hilltop_fs.msh.gz"), "wb", mtime=0) as dst:
        dst.write(data)
    cfg = json.load(open(os.path.join(ref, "cases/2d_hilltop/2d_hilltop.json")))
    cfg["mesh"]["File"] = "2d_hilltop_fs.msh"
    with open(os.path.join(HERE, "2d_hilltop.json"), "w") as f:
        json.dump(cfg, f, indent=1)
    with open(os.path.join(ref, "doc/1d/line.msh"), "rb") as src, open(os.path.join(HERE, "line_1d.msh"), "wb") as dst:
        dst.write(src.read())


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of a checkout of the reference>")
    main(sys.argv[1])
