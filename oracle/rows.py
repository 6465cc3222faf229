"""Row runs to visibility samples: CPU restatement (test infrastructure).

Restates, in numpy with float32 arithmetic where the reference uses f32:
  * routed_weighted_grid_sample_from_run (casa-imaging lib.rs:880-1062): per
    (row, channel) one explicit correlation or a collapsed pair of parallel
    hands, dropped when a used correlation is flagged, the visibility is not
    finite, a weight is not finite and positive, or the sumwt factor is not;
    a pair's natural weight is 0.5 * (w1 + w2) in f32;
  * collapse_standard_mfs_pair_visibility (execution.rs:2323-2340) with
    num-complex's operations (Complex32 * f32 scales both parts; the complex
    product is (a c - b d, a d + b c), unfused);
  * casa_vis_imaging_weight_uv_lambda (weighting.rs:748-756): the density
    coordinates f64(f32(u_m * f64(f32(f / c))));
  * derive_pair_selection / paired_sumwt_factor (types.rs:62-138).
Pinned by the reference's own KATs (lib.rs:88688-88726): a flagged hand
drops the sample; (2+1i, 6-1i) with weights (1.5, 3) collapses to Stokes I
4+0i with weight 2.25 and sumwt factor 2.
"""
import numpy as np

f32 = np.float32

TRANSFORMS = ("half_sum", "half_difference", "positive_half_imag_difference",
              "negative_half_imag_difference")


def collapse(a: complex, b: complex, transform: str) -> complex:
    ar, ai, br, bi = f32(a.real), f32(a.imag), f32(b.real), f32(b.imag)
    if transform == "half_sum":
        return complex(f32(f32(ar + br) * f32(0.5)), f32(f32(ai + bi) * f32(0.5)))
    dr, di = f32(ar - br), f32(ai - bi)
    if transform == "half_difference":
        return complex(f32(dr * f32(0.5)), f32(di * f32(0.5)))
    s = f32(0.5) if transform == "positive_half_imag_difference" else f32(-0.5)
    return complex(f32(f32(dr * f32(0.0)) - f32(di * s)), f32(f32(dr * s) + f32(di * f32(0.0))))


def plane_polarization(plane: str, corr_types):
    """(corr0, corr1 or None, transform, sumwt_factor) for a plane."""
    idx = {c: k for k, c in reversed(list(enumerate(corr_types)))}
    pair = lambda a, b: (idx[a], idx[b]) if a in idx and b in idx else None
    xx_yy, xy_yx, rr_ll, rl_lr = pair(9, 12), pair(10, 11), pair(5, 8), pair(6, 7)
    factor = 2.0 if plane == "I" else 1.0
    choices = {"I": [(xx_yy, "half_sum"), (rr_ll, "half_sum")],
               "Q": [(xx_yy, "half_difference"), (rl_lr, "half_sum")],
               "U": [(xy_yx, "half_sum"), (rl_lr, "positive_half_imag_difference")],
               "V": [(xy_yx, "negative_half_imag_difference"), (rr_ll, "half_difference")]}
    if plane in choices:
        for p, t in choices[plane]:
            if p is not None:
                return p[0], p[1], t, factor
        raise ValueError("the correlations cannot form this plane")
    code = {"XX": 9, "YY": 12, "RR": 5, "LL": 8}[plane]
    if code not in idx:
        raise ValueError("the correlations cannot form this plane")
    return idx[code], None, "half_sum", 1.0


def prepare(uvw_m, lambda_scale, data, flag, weight, spectrum, gridable, corr0, corr1,
            transform, sumwt_factor):
    """Kept (row, channel) samples in that order: dict of u, v, w, weight,
    sumwt_factor, gridable, vis, du, dv."""
    R, C, K = data.shape
    out = {k: [] for k in ("u", "v", "w", "weight", "sumwt_factor", "gridable", "vis", "du",
                           "dv")}
    sf = f32(sumwt_factor)
    ok_pos = lambda x: bool(np.isfinite(x) and x > 0)
    for r in range(R):
        for c in range(C):
            if not ok_pos(sf):
                continue
            wt = (lambda k: f32(spectrum[r, c, k])) if spectrum is not None else \
                (lambda k: f32(weight[r, k]))
            fl = (lambda k: bool(flag[r, c, k])) if flag is not None else (lambda k: False)
            if corr1 is None:
                if fl(corr0):
                    continue
                vis = complex(data[r, c, corr0])
                if not (np.isfinite(vis.real) and np.isfinite(vis.imag)):
                    continue
                natural = wt(corr0)
            else:
                if fl(corr0) or fl(corr1):
                    continue
                vis = collapse(complex(data[r, c, corr0]), complex(data[r, c, corr1]), transform)
                if not (np.isfinite(vis.real) and np.isfinite(vis.imag)):
                    continue
                w0, w1 = wt(corr0), wt(corr1)
                if not (ok_pos(w0) and ok_pos(w1)):
                    continue
                natural = f32(f32(0.5) * f32(w0 + w1))
            if not ok_pos(natural):
                continue
            ls = float(lambda_scale[c])
            ls32 = float(f32(ls))
            um, vm, wm = (float(x) for x in uvw_m[r])
            out["u"].append(um * ls)
            out["v"].append(vm * ls)
            out["w"].append(wm * ls)
            out["du"].append(float(f32(um * ls32)))
            out["dv"].append(float(f32(vm * ls32)))
            out["weight"].append(natural)
            out["sumwt_factor"].append(sf)
            out["gridable"].append(1 if gridable is None or gridable[r] else 0)
            out["vis"].append(vis)
    return {"u": np.array(out["u"], np.float64), "v": np.array(out["v"], np.float64),
            "w": np.array(out["w"], np.float64), "du": np.array(out["du"], np.float64),
            "dv": np.array(out["dv"], np.float64),
            "weight": np.array(out["weight"], np.float32),
            "sumwt_factor": np.array(out["sumwt_factor"], np.float32),
            "gridable": np.array(out["gridable"], np.uint8),
            "vis": np.array(out["vis"], np.complex64)}
