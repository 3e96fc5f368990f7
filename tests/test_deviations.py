"""How far the documented departures of the oracle (and of libvmr, which
follows it bit for bit) move a rendered image from the reference's.

Vec3Normalize.  The reference's amd64 build normalises with an RSQRTSS
estimate refined by one Newton step (math/vec3_amd64.s:11-42); the estimate
is the processor's and differs between processor families (Intel documents
a relative error below 1.5 * 2^-12).  The oracle can emulate that code: an
estimate drawn within the documented bound (a hash of the input and a seed
stands in for the processor's table), then the assembly's Newton step in
its operation order.  Rendering the small-room configuration as configured
(256x256, 16 iterations, 16,384 triangles) with the exact normalisation and
with two emulated estimators bounds what the departure does to an image; it
must stay inside the benchmark spec's tolerance: mean relative pixel error <=
1e-3.  Per pixel: the 99th percentile is asserted <= 1e-3 and at most 1%
of the pixels may move by more than 5%; those are pixels where a camera or
shadow ray whose direction moved by an ulp meets a different soup triangle
at an edge, which changes one of the pixel's 16 samples (observed: median
7.8e-6, 99th percentile 1.8e-4, 0.4% of pixels above 5%, maximum 1.18).

The figures are printed (pytest -s) and recorded in the design notes.
"""
import numpy as np

from vermeer_gb300 import scenes

MEAN_REL = 1e-3
P99_REL = 1e-3
FRAC_ABOVE_5PCT = 0.01


def _pixel_rel(a, b):
    return np.abs(a - b).sum(-1) / np.maximum(np.abs(b).sum(-1), 1e-3)


def test_rsqrtss_normalize_moves_the_small_room_within_tolerance(orc):
    room = scenes.small_room(16384, seed=1, res=256)
    r = orc.Render(room)
    try:
        orc.set_normalize_mode(0)
        exact = r.run(256, 256, 0, 16, 1)
        for seed in (1, 2):
            orc.set_normalize_mode(1, seed)
            emu = r.run(256, 256, 0, 16, 1)
            rel = _pixel_rel(emu, exact)
            changed = (np.abs(emu - exact).max(-1) > 0).mean()
            p50, p99 = np.percentile(rel, [50, 99])
            above = (rel > 0.05).mean()
            print(f"RSQRTSS emulation seed {seed}: mean relative pixel error {rel.mean():.3e}, median {p50:.2e}, "
                  f"99th percentile {p99:.2e}, above 5% {above:.4f}, max {rel.max():.3f}, "
                  f"pixels changed {changed:.3f}")
            assert not np.array_equal(emu, exact)  # the emulation is live
            assert rel.mean() <= MEAN_REL
            assert p99 <= P99_REL
            assert above <= FRAC_ABOVE_5PCT
    finally:
        orc.set_normalize_mode(0)
