"""Shared helpers of the GPU parity tests."""
import numpy as np

from conftest import ANGLE_THRESH, DIST_THRESH, TOLERANCE_REPORT

# Pose tolerance against the oracle: 1e-5 rad / 1e-5 m, the bound the
# reference path is held to.  It is widened only for inputs on which the
# reference algorithm itself does not determine the pose to that precision:
# where the oracle's FP32 and FP64 runs differ by GAP_LIMIT or more.
POSE_TOL_RAD = 1e-5
POSE_TOL_M = 1e-5
GAP_LIMIT = 5e-6


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def dev_u16(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda().view(torch.uint16)


def new_gpu_odo(cam):
    from slam_gb300 import RGBDOdometry
    return RGBDOdometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DIST_THRESH, ANGLE_THRESH)


def new_oracle_odo(cam, prec=32):
    from oracle import oracle
    return oracle.Odometry(cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy, DIST_THRESH, ANGLE_THRESH,
                           prec=prec)


def load_frame(odo, pair, first=True):
    """The reference call order (src/apps/elastic_fusion_file.cpp:359-374)."""
    is_gpu = hasattr(odo, "handle")
    cv = dev if is_gpu else (lambda a: a)
    cd = dev_u16 if is_gpu else (lambda a: a)
    if first:
        odo.initFirstRGB(cv(pair["prev_rgba"]))
    odo.initICPModel(cv(pair["model_vert"]), cv(pair["model_norm"]), 20.0, pair["T1"].astype(np.float32))
    odo.initRGBModel(cv(pair["model_rgba"]))
    odo.initICP(cd(pair["depth"]), 20.0)
    odo.initRGB(cv(pair["rgba"]))


def track(odo, pair, **kw):
    T1 = pair["T1"]
    args = dict(rgbOnly=False, icpWeight=10.0, pyramid=True, fastOdom=False, so3=True)
    args.update(kw)
    t, R = odo.getIncrementalTransformation(T1[:3, 3].astype(np.float32), T1[:3, :3].astype(np.float32), **args)
    return np.asarray(t, np.float64), np.asarray(R, np.float64)


def pose_diff(t1, R1, t2, R2):
    from slam_gb300 import synth
    return synth.pose_error(synth.pose(R1, t1), synth.pose(R2, t2))


def intr(cam, level):
    d = float(1 << level)
    return (float(np.float32(cam.fx) / np.float32(d)), float(np.float32(cam.fy) / np.float32(d)),
            float(np.float32(cam.cx) / np.float32(d)), float(np.float32(cam.cy) / np.float32(d)))


def corr_to_dataterm(corr):
    """GPU correspondence records (u0, v0, diff, valid) -> oracle DataTerm array."""
    from oracle.oracle import DATATERM_DTYPE
    h, w, _ = corr.shape
    out = np.zeros((h, w), DATATERM_DTYPE)
    out["zero_x"] = corr[..., 0]
    out["zero_y"] = corr[..., 1]
    yy, xx = np.mgrid[0:h, 0:w]
    out["one_x"] = xx
    out["one_y"] = yy
    out["diff"] = corr[..., 2].astype(np.float32)
    out["valid"] = corr[..., 3]
    return out


def rel_close(a, b, rtol):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= rtol * scale, float(np.abs(a - b).max() / scale)


def report(line):
    TOLERANCE_REPORT.append(line)
    print(line)


# The integer images of the photometric term (intensity pyramids, derivative
# images).  Their kernels make rounding decisions -- truncations of quotients
# and weighted sums -- that the reference takes with its approximate
# division; the CPU oracle takes them with IEEE arithmetic and differs on tie
# pixels.  Ours match the reference's kernels bit for bit
# (test_gpu_reference.py), so whole-tracking comparisons give the oracle's
# host loop these images from the GPU: what remains between the two is the
# tracking loop itself.
IMAGE_BUFFERS = (("lastImage", 7), ("nextImage", 8), ("lastNextImage", 9), ("dIdx", 10), ("dIdy", 11))


def gpu_images(g):
    """The reference-exact integer images of a loaded GPU handle (derivatives
    computed from its nextImage, as the tracking call does)."""
    g.debug_derivatives()
    return {(name, l): g.download(which, l) for name, which in IMAGE_BUFFERS for l in range(3)}


def pair_images(pair, first=True):
    """gpu_images of a frame pair loaded on a fresh GPU handle."""
    g = new_gpu_odo(pair["cam"])
    load_frame(g, pair, first)
    out = gpu_images(g)
    g.close()
    return out


def set_images(o, images):
    for (name, l), a in images.items():
        o.set_buffer(name, l, a)
    o.keep_derivatives(True)


# How precisely the reference algorithm determines the pose on an input is
# measured by perturbing the oracle's own run: its FP64 twin (precision);
# flagged rounding ties decided the other way -- all of them, and each half
# of them under four hashed splits (the decisions the reference's approximate
# division and square root may take differently from the oracle's IEEE
# arithmetic; the GPU's kernels, which equal the reference's, take some
# subset of them differently); two other summation orders of every pairwise
# sum (reversed; split at a third -- the GPU's reduction tree is another
# order again); and, when a loop decision (the SO3 convergence and
# divergence tests, the rgbOnly early exit) compared two values within
# DECISION_MARGIN, that decision taken the other way.  A GPU pose passes when
# it is within 1e-5 of the oracle's, or within 1e-5 of one of the perturbed
# FP32 runs (it took that run's decisions), or within twice the sum of the
# precision, tie (largest), order (largest) and decision differences, all of
# which must be below GAP_LIMIT for the flat bound alone to apply.  Where one
# exceeds UNDETERMINED (1 cm / 10 mrad) the algorithm does not determine the
# pose on this input (e.g. ICP alone diverging from a large motion): the pose
# is only required to be finite, and the case is reported.
UNDETERMINED = 1e-2
DECISION_MARGIN = 1e-3
TIE_SPLITS = 4
PERTURBATIONS = {"fp64": (64, None), "ties": (32, 1)}
for _k in range(2 * TIE_SPLITS):
    PERTURBATIONS["ties_%d" % _k] = (32, 2 + _k)
PERTURBATIONS.update({"order": (32, "reverse"), "order_b": (32, "third"), "decision": (32, "decision")})
TIE_RUNS = ["ties"] + ["ties_%d" % k for k in range(2 * TIE_SPLITS)]


class OracleRuns:
    """The oracle's host loop on one tracking input, run on demand: FP32 (the
    comparison) and its perturbations.  load(o) puts the inputs into a fresh
    oracle handle (the call order of the caller); start = (t, R) the start
    pose; levels / iterations the batched tracker's per-pair schedule (0: the
    reference's)."""

    def __init__(self, cam, load, start, flags, levels=0, iterations=(0, 0, 0)):
        self.cam, self.load, self.start, self.flags = cam, load, start, dict(flags)
        self.levels, self.iterations = levels, iterations
        self._runs = {}

    def run(self, prec=32, perturb=None):
        """perturb: None; 1 (every tie the other way) or m >= 2 (half (m - 2) % 2
        of the ties under hashed split (m - 2) / 2); "reverse" / "third" (other
        summation orders); "decision" (the closest loop decision of the
        unperturbed run the other way)."""
        key = (prec, perturb)
        if key not in self._runs:
            from oracle import oracle
            flip_decision = self.run(prec)[2].decision_margin()[1] if perturb == "decision" else None

            def once():
                o = new_oracle_odo(self.cam, prec)
                if self.levels:
                    o.set_schedule(self.levels, self.iterations)
                self.load(o)
                if flip_decision is not None:
                    o.set_flip_decision(flip_decision)
                oracle.set_flip_ties(prec, perturb if isinstance(perturb, int) else 0)
                oracle.set_reverse_sums(prec, {"reverse": 1, "third": 2}.get(perturb, 0))
                try:
                    t, R = o.getIncrementalTransformation(np.float32(self.start[0]).astype(o.k.real),
                                                          np.float32(self.start[1]).astype(o.k.real), **self.flags)
                finally:
                    oracle.set_flip_ties(prec, 0)
                    oracle.set_reverse_sums(prec, 0)
                return np.asarray(t, np.float64), np.asarray(R, np.float64), o

            self._runs[key] = once()
        return self._runs[key]

    @property
    def main(self):
        return self.run(32)

    def near_decision(self):
        m, idx = self.run(32)[2].decision_margin()
        return idx >= 0 and m < DECISION_MARGIN

    def _perturbed(self):
        return [k for k in PERTURBATIONS if k != "decision" or self.near_decision()]

    def sensitivity(self):
        """{name: (rad, m)} differences of the perturbed runs from the FP32 run."""
        t32, R32, _ = self.run(32)
        out = {}
        for name in self._perturbed():
            t, R, _ = self.run(*PERTURBATIONS[name])
            out[name] = pose_diff(t32, R32, t, R)
        return out

    def summation_gap(self):
        """Largest pose change (rad or m) of the oracle's own result under the
        perturbations that are properties of the reference algorithm rather
        than of the oracle's IEEE arithmetic: another summation order (the
        reference's depends on its launch shape) and FP64 arithmetic."""
        t32, R32, _ = self.run(32)
        return max(max(pose_diff(t32, R32, *self.run(*PERTURBATIONS[k])[:2])) for k in ("order", "order_b", "fp64"))

    def undetermined(self):
        worst = max(max(v) for v in self.sensitivity().values())
        return not np.isfinite(worst) or worst > UNDETERMINED

    def tolerance(self):
        """(tol_rad, tol_m, how); tol = inf for an undetermined input."""
        s = self.sensitivity()
        how = ", ".join("%s %.1e rad %.1e m" % (k, v[0], v[1]) for k, v in s.items())
        worst = max(max(v) for v in s.values())
        if not np.isfinite(worst) or worst > UNDETERMINED:
            return float("inf"), float("inf"), "undetermined (" + how + ")"
        if worst < GAP_LIMIT:
            return POSE_TOL_RAD, POSE_TOL_M, "flat (" + how + ")"
        tie = [max(s[k][i] for k in TIE_RUNS) for i in (0, 1)]
        order = [max(s["order"][i], s["order_b"][i]) for i in (0, 1)]
        tol = [2 * (s["fp64"][i] + tie[i] + order[i] + (s["decision"][i] if "decision" in s else 0.0))
               for i in (0, 1)]
        return max(POSE_TOL_RAD, tol[0]), max(POSE_TOL_M, tol[1]), "widened (" + how + ")"

    def iterations_ok(self, gpu_iterations):
        """The GPU's iteration counts equal the oracle's or those of one of
        its FP32 perturbations (a near-tie loop decision may stop a loop one
        iteration earlier or later)."""
        runs = [self.run(32)] + [self.run(*PERTURBATIONS[k]) for k in self._perturbed() if k != "fp64"]
        return any(list(gpu_iterations) == r[2].iterations() for r in runs)

    def spread(self, metric):
        """Twice the combined change of metric(oracle handle) (a scalar) under
        the perturbations: precision + ties (largest of the three) + order +
        decision, as the pose bound combines them."""
        base = metric(self.run(32)[2])
        d = {k: abs(metric(self.run(*PERTURBATIONS[k])[2]) - base) for k in self._perturbed()}
        tie = max(d[k] for k in TIE_RUNS)
        return 2 * (d["fp64"] + tie + max(d["order"], d["order_b"]) + d.get("decision", 0.0))

    def jtj_tolerance(self, flat):
        """Relative tolerance of lastA (max-normalised): 1e-3 (sums of
        ~1e4-1e5 FP32 products in another order) where the pose is within the
        flat bound, else also the combined spread of lastA."""
        if flat:
            return 1e-3
        A = self.run(32)[2].stats["lastA"]
        scale = max(np.abs(A).max(), 1e-30)
        return max(1e-3, max(self.spread(lambda o, i=i: o.stats["lastA"].reshape(-1)[i]) for i in range(36)) / scale)

    def _fp32_runs(self):
        return [("main", self.run(32))] + [(k, self.run(*PERTURBATIONS[k])) for k in self._perturbed() if k != "fp64"]

    def matches_a_tie_run(self, tg, Rg):
        """True when the GPU pose is within the flat 1e-5 of one of the oracle
        runs whose flagged rounding ties were decided the other way (the GPU
        took a set of tie decisions the oracle's IEEE arithmetic takes
        differently)."""
        for k in TIE_RUNS:
            t, R, _ = self.run(*PERTURBATIONS[k])
            rot, tr = pose_diff(tg, Rg, t, R)
            if rot <= POSE_TOL_RAD and tr <= POSE_TOL_M:
                return True
        return False

    def closest_run(self, tg, Rg):
        """(name, (rad, m)) of the FP32 run (unperturbed or perturbed) closest
        to a GPU pose."""
        d = [(name, pose_diff(tg, Rg, r[0], r[1])) for name, r in self._fp32_runs()]
        return min(d, key=lambda x: max(x[1][0] / POSE_TOL_RAD, x[1][1] / POSE_TOL_M))

    def jtj_ok(self, A_gpu, flat):
        """(ok, err): lastA within 1e-3 of the oracle's (max-normalised relative
        difference err; sums of ~1e4-1e5 FP32 products in another order and
        the odd tie pixel), else within the combined spread of lastA under the
        perturbations, or within 1e-3 of the lastA of one of the perturbed FP32
        runs (the GPU took that run's decisions)."""
        A_gpu = np.asarray(A_gpu, np.float64).reshape(6, 6)
        rel = lambda A: float(np.abs(A_gpu - A).max() / max(np.abs(A).max(), 1e-30))
        err = rel(self.run(32)[2].stats["lastA"])
        if err <= 1e-3 or err <= self.jtj_tolerance(False):
            return True, err
        return any(rel(r[2].stats["lastA"]) <= 1e-3 for _, r in self._fp32_runs()), err

    def count_ok(self, name, value, flat):
        """A final count within count_tolerance of the oracle's, or within
        0.2 % of one of the perturbed FP32 runs' counts."""
        if abs(value - self.run(32)[2].stats[name]) <= self.count_tolerance(name, flat):
            return True
        return any(abs(value - r[2].stats[name]) <= 0.002 * max(1.0, r[2].stats[name]) for _, r in self._fp32_runs())

    def count_tolerance(self, name, flat):
        """Tolerance of a final inlier / correspondence count ("lastICPCount",
        "lastRGBCount"): 0.2 % (per-pixel decisions on rounding ties) where the
        pose is within the flat bound, else also its combined spread."""
        base = max(1.0, self.run(32)[2].stats[name])
        return 0.002 * base if flat else max(0.002 * base, self.spread(lambda o: o.stats[name]))


def frame_runs(pair, flags, levels=0, iterations=(0, 0, 0), first=True, images=None):
    """OracleRuns of a frame pair loaded in the reference's call order (with
    the GPU's integer images when given), started from pair["T1"]."""
    def load(o):
        load_frame(o, pair, first)
        if images is not None:
            set_images(o, images)
    T1 = pair["T1"]
    return OracleRuns(pair["cam"], load, (T1[:3, 3], T1[:3, :3]), flags, levels, iterations)


def oracle_track(pair, flags, levels=0, iterations=(0, 0, 0), prec=32, first=True, images=None):
    """The oracle's host loop on one pair.  Returns (t, R, oracle handle)."""
    return frame_runs(pair, flags, levels, iterations, first, images).run(prec)


def check_pose(label, tg, Rg, to, Ro, tol_fn):
    """Asserts that the GPU pose is within tolerance of the oracle's and
    records the tolerance applied.  A pose within the flat 1e-5 bound passes
    as it is; otherwise tol_fn() -> (tol_rad, tol_m, how) gives the bound for
    this input (OracleRuns.tolerance)."""
    rot, tr = pose_diff(tg, Rg, to, Ro)
    if rot <= POSE_TOL_RAD and tr <= POSE_TOL_M:
        report("%s: pose diff %.2e rad %.2e m <= flat 1e-5" % (label, rot, tr))
        return rot, tr, True
    tol_r, tol_t, how = tol_fn()
    assert np.all(np.isfinite(tg)) and np.all(np.isfinite(Rg)), label
    owner = getattr(tol_fn, "__self__", None)
    if not (rot <= tol_r and tr <= tol_t) and isinstance(owner, OracleRuns):
        name, d = owner.closest_run(tg, Rg)
        if d[0] <= POSE_TOL_RAD and d[1] <= POSE_TOL_M:
            report("%s: pose diff %.2e rad %.2e m; within the flat 1e-5 of the oracle run with %s perturbed "
                   "(%.2e rad %.2e m)" % (label, rot, tr, name, d[0], d[1]))
            return rot, tr, False
    report("%s: pose diff %.2e rad %.2e m, tolerance %.2e rad %.2e m %s" % (label, rot, tr, tol_r, tol_t, how))
    assert rot <= tol_r and tr <= tol_t, (label, rot, tr, tol_r, tol_t, how)
    return rot, tr, False
