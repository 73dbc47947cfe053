"""Command line for the DMC path (the reference's GUI actions, headless):

  python -m manifolddmc_gb300.cli run volume.bin --iso 900 [--refine R] [--pad]
        [--no-split] [--no-detect] [--no-surface-iteration] [--simplify3x3y]
        [--simplify3x3y-old] [--simplify3333] --obj out.obj [--stats Statistics.json]
        [--color-faces] [--quality qualityDMC.bin]
  python -m manifolddmc_gb300.cli mc volume.bin --iso 900 [--refine R] [--pad] [--obj out.obj]
        [--quality qualityMC.bin]
  python -m manifolddmc_gb300.cli generate sphere --dims 64 64 64 --bin out.bin [--scale 1000]
  python -m manifolddmc_gb300.cli check mesh.obj
  python -m manifolddmc_gb300.cli canonical in.obj out.obj
"""
import argparse
import json
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser(prog="manifolddmc_gb300.cli")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run")
    r.add_argument("volume")
    r.add_argument("--iso", type=float, required=True)
    r.add_argument("--refine", type=int, default=0)
    r.add_argument("--pad", action="store_true")
    r.add_argument("--no-split", action="store_true")
    r.add_argument("--no-detect", action="store_true")
    r.add_argument("--no-surface-iteration", action="store_true")
    r.add_argument("--simplify3x3y", action="store_true")
    r.add_argument("--simplify3x3y-old", action="store_true")
    r.add_argument("--simplify3333", action="store_true")
    r.add_argument("--obj")
    r.add_argument("--stats")
    r.add_argument("--color-faces", action="store_true", help="reduce the face colors to 5 (FaceColoring.cu)")
    r.add_argument("--quality", help="mean-ratio quality of the quads' triangles, int32 count + float32 each")
    m = sub.add_parser("mc")
    m.add_argument("volume")
    m.add_argument("--iso", type=float, required=True)
    m.add_argument("--refine", type=int, default=0)
    m.add_argument("--pad", action="store_true")
    m.add_argument("--obj")
    m.add_argument("--quality")
    g = sub.add_parser("generate")
    g.add_argument("surface")
    g.add_argument("--dims", type=int, nargs=3, default=[64, 64, 64])
    g.add_argument("--bin", required=True)
    g.add_argument("--scale", type=float, default=1000.0, help="value = scale * f + offset, stored as uint16")
    g.add_argument("--offset", type=float, default=1000.0)
    c = sub.add_parser("check")
    c.add_argument("obj")
    k = sub.add_parser("canonical")
    k.add_argument("obj")
    k.add_argument("out")
    a = ap.parse_args(argv)

    from . import meshtools
    if a.cmd == "check":
        pos, quads = meshtools.read_obj(a.obj)
        print(json.dumps(meshtools.manifold_report(quads, len(pos))))
        return 0
    if a.cmd == "canonical":
        pos, quads = meshtools.read_obj(a.obj)
        meshtools.write_obj(a.out, *meshtools.canonicalize(pos, quads))
        return 0
    import manifolddmc_gb300 as mdmc
    if a.cmd == "generate":
        vol, origin, spacing = mdmc.generate_volume(a.surface, a.dims)
        mdmc.write_bin(a.bin, vol.cpu().numpy() * np.float32(a.scale) + np.float32(a.offset), spacing)
        return 0
    if a.cmd == "mc":
        import torch
        dmc = mdmc.DualMarchingCubes()
        grid = mdmc.UniformGrid.read_from_file(a.volume, a.refine, a.pad)
        pos, nrm, tri = dmc.run_standard_mc(a.iso, grid)
        if a.obj:
            # the older CLI's mesh copy negates the gradient normals
            # (OriginalDMC/src/DualMarchingCubes.cu:1034)
            meshtools.write_triangle_obj(a.obj, pos, -nrm, tri)
        if a.quality:
            q = mdmc.mean_ratio(torch.from_numpy(pos).cuda(), torch.from_numpy(tri).cuda())
            meshtools.write_quality_bin(a.quality, q.cpu().numpy())
        print(json.dumps({"vertices": len(pos), "triangles": len(tri)}))
        return 0
    dmc = mdmc.DualMarchingCubes(
        split_non_manifold_halfedges=int(not a.no_split), detect_non_manifold_vertices=int(not a.no_detect),
        enable_surface_to_vertex_iteration=int(not a.no_surface_iteration), simplify_p3x3y_color=int(a.simplify3x3y),
        simplify_p3x3y_old=int(a.simplify3x3y_old), simplify_p3333=int(a.simplify3333))
    grid = mdmc.UniformGrid.read_from_file(a.volume, a.refine, a.pad)
    times = dmc.run(a.iso, grid)
    if a.color_faces:
        dmc.color_faces()
    if a.obj:
        dmc.write_obj(a.obj)
    if a.quality:
        dev = dmc.device_arrays()
        q = mdmc.mean_ratio(dev["positions"], mdmc.quads_to_triangles(dev["quads"]))
        meshtools.write_quality_bin(a.quality, q.cpu().numpy())
    if a.stats:
        meshtools.append_statistics(a.stats, meshtools.statistics_record(
            a.volume, grid.dimensions, a.iso, dmc.stats, int(dmc.mesh.num_vertices)))
    print(json.dumps({"vertices": int(dmc.mesh.num_vertices), "faces": int(dmc.mesh.num_faces),
                      "edges4": dmc.get_num_non_manifold_edges4(), "ms": times}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
