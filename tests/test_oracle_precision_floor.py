"""What bounds the colours of the precision form, measured on the oracle (CPU only).

The precision form keeps the moment image and the re-march in FP32 and computes only the moment sums (Kahan) and
the Lagrange multipliers (FP64 / float-float) with more precision.  On a 64-moment mixing-layer image this test
rounds one quantity at a time to float around an all-FP64 evaluation of the same method and measures the RGBA
change:
  * the re-march in FP32, fed the FP64 multipliers (rounded to float, as the FP32 re-march reads them);
  * the multipliers alone rounded to float, the re-march in FP64;
  * the moments alone rounded to float, the preparation and the re-march in FP64.
Each alone moves some pixels by more than 1e-3: the MESE series sum_l lambda_l cos(l theta) cancels terms of up to
|lambda| ~ 1e4 to values of order one.  So an FP32 re-march puts a floor far above 1e-4 under the RGBA error of any
form that keeps it, whatever precision the moments and the multipliers carry.
"""
import numpy as np

import oracle as O


def test_fp32_remarch_bounds_the_precision_form():
    from mray_gb300 import workloads as W

    n, size, m = 128, 128, 64
    wl = W.mixing_layer_workload(n=n, width=size, height=size, num_moments=m)
    mom, bounds, counts = O.generate_moments(wl.camera, wl.gen, wl.volume, wl.domain_min, wl.domain_max, size, size,
                                             m, "f64")
    table = O.preintegrate(wl.tf1d, wl.tf_step)
    index, _ = O.compact(counts, mom.astype(np.float32))
    data = mom.reshape(-1, m)[counts.reshape(-1) > 0].reshape(-1)

    def prep(d):
        return O.prepare_moments(size, size, m, index, d, bias=wl.rec.bias, precision="f64")

    def rec(pm, precision):
        return O.reconstruct(wl.camera, wl.rec, size, size, m, wl.domain_min, wl.domain_max, index, pm, bounds,
                             table, precision)

    pm = prep(data)
    ref = rec(pm, "f64")
    remarch32 = np.abs(rec(pm.astype(np.float32), "f32") - ref).max()
    lambda32 = np.abs(rec(pm.astype(np.float32).astype(np.float64), "f64") - ref).max()
    moments32 = np.abs(rec(prep(data.astype(np.float32).astype(np.float64)), "f64") - ref).max()
    print(f"max |dRGBA| against all-FP64: FP32 re-march {remarch32:.2e}, multipliers rounded {lambda32:.2e}, "
          f"moments rounded {moments32:.2e}")
    assert remarch32 > 1e-3
    assert lambda32 > 1e-3
    assert moments32 > 1e-3
