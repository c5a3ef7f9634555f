"""A small, self-contained profiling case: one Tb.Th and one Tb.Sp local
thickness of a seeded n^3 specimen (sigma 5, BV/TV 0.15, cylinder ROI of
radius 0.47 n, the 512^3 workload's generator at a smaller edge; with
``plates``, the 1024^3 workload's generator: sigma (4, 4, 8), BV/TV 0.30,
sphere ROI of radius 500 n / 1024).

Run as ``python -m bone_morphometry_gb300.profile_case [n] [plates]`` under a profiler
with a kernel filter; the first call builds the search-template tables and is
a warm-up, the next two are the launches worth capturing (Tb.Th then Tb.Sp).
"""

from __future__ import annotations

import sys


def main(argv=None) -> int:
    import numpy as np
    import torch

    from . import Context, Phase, local_thickness
    from . import synthetic as S

    argv = sys.argv[1:] if argv is None else argv
    n = int(argv[0]) if argv else 256
    if len(argv) > 1 and argv[1] == "plates":
        sp = S.make_specimen_torch((n, n, n), (4.0, 4.0, 8.0), 0.30, "sphere", 500.0 * n / 1024, 8.0, 1003,
                                   to_host=True)
    else:
        sp = S.make_specimen((n, n, n), 5.0, 0.15, "cylinder", 0.47 * n, 19.5, 1002)
    ctx = Context(0)
    th = torch.from_numpy(((sp.roi != 0) & (sp.bone != 0)).astype(np.uint8)).cuda()
    ma = torch.from_numpy(((sp.roi != 0) & (sp.bone == 0)).astype(np.uint8)).cuda()
    local_thickness(th, Phase.FOREGROUND, ctx=ctx)
    local_thickness(th, Phase.FOREGROUND, ctx=ctx)
    local_thickness(ma, Phase.FOREGROUND, ctx=ctx)
    torch.cuda.synchronize()
    print("profile case done: %d^3 %s" % (n, " ".join(argv[1:])))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
