"""Command-line drivers with the reference's parameter conventions.

The reference's programs take SEP parameters as key=value arguments, or as
a JSON object through json=<file> (scripts/run.py:38-49, :66-74).  Here:

  python sc17-born_gb300/cli.py add in1=a.json in2=b.json out=c.json
      util/Add (util/Add.cc): out = in1 + in2 for SEP or JSON regular files.

  python sc17-born_gb300/cli.py rtm data=d.H wavelet=w.H velocity=v.H \\
      image=img.json [src_depth=20 rec_depth=10 nbound=50]
      RTM3D (rtm.cc:10-41): the RTM image of every shot of the data file,
      summed, through the Born operator on the GPU (rtm_zero_op's adjoint,
      reference mode).  The data file's axes are those data_rtm_3d and
      rtm.cc read (data_rtm_3d.cc:4-28, rtm.cc:23-26): 1 time, 2 and 3 the
      receiver x and y, 4 and 5 the source x and y (a source at every
      pair).  The image has the velocity's grid.  Under torchrun (one rank
      per GPU) each rank migrates the shots r, r + W, ... and the images are
      summed over the ranks on the devices before rank 0 writes the file: the
      in-process form of the reference's shot farm (scripts/run.py), whose
      Add step is the all-reduce.
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def package():
    if "born_gb300" in sys.modules:
        return sys.modules["born_gb300"]
    spec = importlib.util.spec_from_file_location(
        "born_gb300", os.path.join(HERE, "__init__.py"),
        submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["born_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def parse_params(argv):
    """key=value arguments; json=<file> merges a JSON object's keys (later
    arguments override earlier ones, as in SEP parameter parsing)."""
    pars = {}
    for a in argv:
        if "=" not in a:
            raise SystemExit(f"argument '{a}' is not key=value")
        k, v = a.split("=", 1)
        if k == "json":
            with open(v) as f:
                obj = json.load(f)
            pars.update({str(kk): str(vv) for kk, vv in obj.items()})
        else:
            pars[k] = v
    return pars


def need(pars, key):
    if key not in pars:
        raise SystemExit(f"missing parameter {key}=")
    return pars[key]


def cmd_add(pars):
    born = package()
    born.add_regfiles(need(pars, "in1"), need(pars, "in2"),
                      need(pars, "out"))
    return 0


def shots_of_rank(nshots, rank, world):
    """Round-robin split of the shots over the ranks (scripts/split.py)."""
    return list(range(rank, nshots, world))


def cmd_rtm(pars, rank=0, world=1):
    image, vo, vd = migrate(pars, rank, world)
    if rank == 0:
        package().write_regfile(need(pars, "image"), image, vo, vd)
    return 0


def migrate(pars, rank=0, world=1):
    """The summed RTM image of this rank's shots (of all ranks' shots when a
    process group of world ranks is running); returns (image, o, d)."""
    born = package()
    data, do, dd = born.read_regfile(need(pars, "data"))
    if data.ndim == 3:  # one shot: its position from sx=, sy=
        data = data[None, None]
        do = tuple(do) + (float(need(pars, "sx")), float(need(pars, "sy")))
        dd = tuple(dd) + (1.0, 1.0)
    if data.ndim != 5:
        raise SystemExit("data must have axes t, rx, ry (one shot, with "
                         "sx=, sy=) or t, rx, ry, sx, sy")
    wav, wo, wd = born.read_regfile(need(pars, "wavelet"))
    vel, vo, vd = born.read_regfile(need(pars, "velocity"))
    if vel.ndim != 3:
        raise SystemExit("velocity must be 3-D")
    nsy, nsx, rny, rnx, nt = data.shape
    src_depth = float(pars.get("src_depth", 0.0))
    rec_depth = float(pars.get("rec_depth", 0.0))
    nbound = int(pars.get("nbound", 50))
    shots = np.array([[do[3] + dd[3] * ix, do[4] + dd[4] * iy, src_depth]
                      for iy in range(nsy) for ix in range(nsx)], np.float32)
    traces = data.reshape(nsy * nsx, rny, rnx, nt)
    mine = shots_of_rank(len(shots), rank, world)
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0
    torch.cuda.set_device(dev)
    image = torch.zeros(vel.shape, device=f"cuda:{dev}")
    if mine:
        op = born.BornOperator(
            vel, vo, vd, shots[mine], wav.ravel(), float(wd[0]), nt,
            float(dd[0]), (rnx, rny), (do[1], do[2]), (dd[1], dd[2]),
            rec_depth, nbound, exact=False, device=dev)
        d = torch.from_numpy(np.ascontiguousarray(traces[mine])).to(
            f"cuda:{dev}")
        op.adjoint(False, image, d)
    if world > 1:
        born.stack_tensor(image)
    return image.cpu().numpy(), vo, vd


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv or argv[0] not in ("add", "rtm"):
        print(__doc__)
        return 2
    pars = parse_params(argv[1:])
    if argv[0] == "add":
        return cmd_add(pars)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        return cmd_rtm(pars, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
