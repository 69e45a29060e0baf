"""Command line for the reference's two drivers.

  python -m fanbeamctrecon_tensorflowop_gb300.cli test [--input ./test.fbp]
      test.py end to end: read float32 [-1, 512, 512] slices, FP them with the
      geometry of ``config``, BP and Ram-Lak FBP the sinograms, and write
      test_prj.raw, test_img_BP.raw and test_img_FBP.raw (test.py:17-41).

  python -m fanbeamctrecon_tensorflowop_gb300.cli fdk-generate --index I
      --start-angle DEG --nview N --nslice S [--folder Training] ...
      FDK_generate of FDK/FDK_test_training.py:18-141, batched.

Every slice of a file goes through one batched call per operator; outputs are
float32 in C order, as the reference's ``bytearray(ndarray)`` writes them.
"""
from __future__ import annotations

import argparse
import os
import sys
import time


def _cmd_test(args) -> int:
    from . import utils
    from .rawio import read_binary_dataset, write_raw

    t0 = time.perf_counter()
    img = read_binary_dataset(args.input, [args.dim[0], args.dim[1]])
    nimg = img.shape[0]
    sino = utils.ForwardProjection(img, nimg)
    write_raw(os.path.join(args.out_dir, "test_prj.raw"), sino)
    bp = utils.BackProjection(sino, nimg)
    write_raw(os.path.join(args.out_dir, "test_img_BP.raw"), bp)
    fbp = utils.FilteredBackProjection(sino, nimg)
    write_raw(os.path.join(args.out_dir, "test_img_FBP.raw"), fbp)
    if not args.quiet:
        print(f"{nimg} slice(s): FP {tuple(sino.shape)}, BP and FBP {tuple(fbp.shape)} "
              f"in {time.perf_counter() - t0:.3f} s -> {args.out_dir}")
    return 0


def _cmd_fdk(args) -> int:
    from .fdk_driver import fdk_generate

    t0 = time.perf_counter()
    out = fdk_generate(args.index, args.start_angle, args.nview, args.nslice,
                       folder=args.folder, data_root=args.data_root, save_root=args.save_root,
                       recon_dir=args.recon_dir, chunk=args.chunk)
    if not args.quiet:
        print(f"exam {args.index}: {len(out['index_data'])} slice(s) x 3 sinograms "
              f"reconstructed in {time.perf_counter() - t0:.3f} s")
    return 0


def build_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="python -m fanbeamctrecon_tensorflowop_gb300.cli",
                                 description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("test", help="test.py: FP, BP and FBP of a raw image file")
    t.add_argument("--input", default="./test.fbp", help="float32 [-1, H, W] C-order file")
    t.add_argument("--dim", type=int, nargs=2, default=[512, 512], metavar=("H", "W"))
    t.add_argument("--out-dir", default=".")
    t.add_argument("--quiet", action="store_true")
    t.set_defaults(func=_cmd_test)
    f = sub.add_parser("fdk-generate", help="FDK_generate of the FDK training-data driver")
    f.add_argument("--index", type=int, required=True)
    f.add_argument("--start-angle", type=float, required=True, help="degrees")
    f.add_argument("--nview", type=int, required=True, help="views per rotation (nview_full)")
    f.add_argument("--nslice", type=int, required=True)
    f.add_argument("--folder", default="Training")
    f.add_argument("--data-root", default=".", help="holds <folder>/exam<index>_<ch>.prj")
    f.add_argument("--save-root", default=".", help="the .npy files go to <save-root>/<folder>")
    f.add_argument("--recon-dir", default="./recon_images")
    f.add_argument("--chunk", type=int, default=96, help="slices per batched call")
    f.add_argument("--quiet", action="store_true")
    f.set_defaults(func=_cmd_fdk)
    return ap


def main(argv=None) -> int:
    args = build_parser().parse_args(argv)
    return args.func(args)


if __name__ == "__main__":
    sys.exit(main())
