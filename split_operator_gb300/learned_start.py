"""Learned starting states for imaginary-time ground-state relaxation.

No counterpart in the reference crate.  Pipeline:

1. Potential parameter sets (D, a, re, beta, mass) -- D in [0.05, 0.2], a in
   [0.6, 1.4], re in [2, 4], beta in [0, 0.05], mass in [500, 2000] -- seeded
   (training: default_rng(5), held out: default_rng(6)).
2. Ground states of V = D (1 - e^{-a(r-re)})^2 + beta e^{-r/2} P2(cos th) on an
   Nr x Ntheta radial x Gauss-Legendre grid, found by the plain FP64 solver:
   imaginary time dt = -i * 1.0, stack [LeakControl(+loss), V/2, Legendre, Rot/2,
   FFT, K], renormalised every step, energies from Propagation::mean_energy, run
   until successive energies differ by <= 1e-10.  Many instances run together
   through the batched executor.
3. A radial basis per l: the leading `modes` left singular vectors of the training
   ground states' radial functions at that l (eigenvectors of their covariance), each
   sampled in the scaled coordinate xi = (r - re) (m omega)^(1/2) of the harmonic
   approximation of its well (cubic splines to and from the radial grid), so that the
   network predicts the shape of the state, not its position and width.
4. A multilayer perceptron (5 -> 256 -> 256 -> 256 -> Ntheta*modes, BF16 weights, FP32
   accumulation) trained on the library's own CUDA kernels to map the scaled
   parameters to the standardised basis coefficients.
5. Held-out evaluation: steps and wall time until |E - E*| <= 1e-8 (E* = the plain
   solver's converged energy) from the learned start and from the plain Gaussian start.

Set-up arithmetic (grids, Legendre matrices, basis) is host numpy; every propagation
and every network product runs in the library's kernels.
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import api as so

PARAM_LO = np.array([0.05, 0.6, 2.0, 0.0, 500.0])
PARAM_HI = np.array([0.2, 1.4, 4.0, 0.05, 2000.0])


def param_sets(count, seed):
    rng = np.random.default_rng(seed)
    return PARAM_LO + (PARAM_HI - PARAM_LO) * rng.uniform(size=(count, 5))


def scale_params(p):
    return (2.0 * (np.asarray(p) - PARAM_LO) / (PARAM_HI - PARAM_LO) - 1.0).astype(np.float32)


def physics_features(p):
    """Five inputs that set the ground state's shape in the well's scaled frame:
    ln lambda (lambda = (2 m D)^(1/2) / a, the Morse anharmonicity: the radial shape in xi
    depends on it alone), ln(1 + q) with q = beta e^(-re/2) 2 m re^2 (the P2 coupling over
    the rotational constant at re: the angular shape), re, ln m and a; each mapped to
    [-1, 1] over the sampled parameter box."""
    p = np.atleast_2d(np.asarray(p, dtype=np.float64))
    d, a, re, beta, m = p.T

    def raw(d, a, re, beta, m):
        lam = np.sqrt(2.0 * m * d) / a
        q = beta * np.exp(-re / 2.0) * 2.0 * m * re * re
        return np.stack([np.log(lam), np.log1p(q), re, np.log(m), a], axis=1)

    # bounds of each feature over the parameter box (its corners hold the extremes:
    # every feature is monotone in each parameter)
    corners = np.array(np.meshgrid(*[[lo, hi] for lo, hi in zip(PARAM_LO, PARAM_HI)])).reshape(5, -1).T
    fc = raw(*corners.T)
    lo, hi = fc.min(axis=0), fc.max(axis=0)
    return (2.0 * (raw(d, a, re, beta, m) - lo) / (hi - lo) - 1.0).astype(np.float32)


class Grid2D:
    """Radial x Gauss-Legendre grid and the Legendre matrices of legendre_diagonalization.rs:13-45."""

    def __init__(self, nr=2048, nth=64, r_min=0.5, r_max=16.5):
        self.nr, self.nth, self.r_min, self.r_max = nr, nth, r_min, r_max
        step = (r_max - r_min) / (nr - 1.0)
        self.r = np.array([r_min + step * i for i in range(nr)])
        self.x, self.w = np.polynomial.legendre.leggauss(nth)
        tinv = np.empty((nth, nth))
        for l in range(nth):
            tinv[:, l] = math.sqrt(l + 0.5) * np.polynomial.legendre.Legendre.basis(l)(self.x)
        self.tinv = tinv                      # theta <- l
        self.t = (tinv * self.w[:, None]).T   # l <- theta

    def to_l(self, psi):  # psi[r, theta] -> psi[r, l]
        return psi @ self.t.T

    def to_theta(self, psi_l):
        return psi_l @ self.tinv.T


def problem(prm, g: Grid2D, psi0=None, precision="fp64"):
    d, a, re, beta, mass = [float(v) for v in prm]
    radial = so.Grid.new_linear_continuos("radial", g.r_min, g.r_max, g.nr, 0)
    polar = so.Grid.new_custom("polar", np.arccos(g.x), g.w, 1)
    r = g.r
    p2 = 0.5 * (3.0 * g.x * g.x - 1.0)
    v = (d * (1.0 - np.exp(-a * (r - re))) ** 2)[:, None] + (beta * np.exp(-r / 2.0))[:, None] * p2[None, :]
    if psi0 is None:
        # plain Gaussian start: isotropic, centred on the well, width 0.5
        psi0 = np.exp(-((r - re) / (2.0 * 0.5)) ** 2)[:, None] * np.ones(g.nth)[None, :]
    wf = so.WaveFunction(np.asarray(psi0, dtype=np.complex128), [radial, polar])
    wf.normalize(1.0)
    tg = so.TimeGrid(1.0, 10 ** 6, True)
    leak = so.LeakControl()
    leak.add_loss_checker("leak control")
    st = so.OperationStack()
    st.add_control(leak, so.FIRST_HALF | so.SECOND_HALF)
    st.add_propagator(so.n_dim_into_propagator(v, tg, so.HALF))
    st.add_transformation(so.legendre_diagonalization_operator(polar), so.NORMAL)
    st.add_propagator(so.n_dim_into_propagator(so.rotational_hamiltonian(radial, polar, mass, 0.0), tg, so.HALF))
    st.add_transformation(so.FFTTransformation(radial, "momentum"), so.NORMAL)
    st.add_propagator(so.one_dim_into_propagator(so.kinetic_hamiltonian(radial, mass), radial, tg, so.FULL))
    return so.Propagation(wf, tg, st, precision)


def relax(props, every=20, max_steps=20000, tol=None, target=None, group=512):
    """Imaginary-time steps until successive energies (every `every` steps) differ by
    <= tol, or until |E - target[i]| <= 1e-8 when `target` is given.  Returns
    (energies, steps incl. the energy evaluations, wall seconds)."""
    n = len(props)
    energy = np.full(n, np.nan)
    prev = np.full(n, np.nan)
    steps = np.zeros(n, dtype=np.int64)
    done = np.zeros(n, dtype=bool)
    t0 = time.perf_counter()
    batches = []  # (member indices, Batch); rebuilt when a quarter of its members finished
    while not done.all():
        active = [i for i in range(n) if not done[i]]
        live = sum(len([i for i in idx if not done[i]]) for idx, _ in batches)
        members = sum(len(idx) for idx, _ in batches)
        if not batches or live < 0.75 * members:
            batches = [(active[s:s + group], so.Batch([props[i] for i in active[s:s + group]]))
                       for s in range(0, len(active), group)]
        for idx, b in batches:
            b.steps(every)  # finished members of a batch keep stepping until it is rebuilt
            for i in idx:
                if done[i]:
                    continue
                steps[i] += every + 1  # mean_energy runs one more step
                e = props[i].mean_energy()
                energy[i] = e
                if target is not None:
                    done[i] = abs(e - target[i]) <= 1e-8
                else:
                    done[i] = np.isfinite(prev[i]) and abs(e - prev[i]) <= tol
                prev[i] = e
                if steps[i] >= max_steps:
                    done[i] = True
    return energy, steps, time.perf_counter() - t0


def ground_states(params, g: Grid2D, tol=1e-10, every=20, max_steps=20000, chunk=512, progress=False):
    """FP64 ground states (real parts, [count, nr, nth]), energies and step counts."""
    states = np.empty((len(params), g.nr, g.nth), dtype=np.float32)
    energies = np.empty(len(params))
    nsteps = np.empty(len(params), dtype=np.int64)
    t0 = time.perf_counter()
    for s in range(0, len(params), chunk):
        if progress:
            print(f"ground states {s}/{len(params)} after {time.perf_counter() - t0:.0f} s", flush=True)
        props = [problem(p, g) for p in params[s:s + chunk]]
        e, st, _ = relax(props, every=every, max_steps=max_steps, tol=tol)
        for k, p in enumerate(props):
            states[s + k] = p.get_array().real
        energies[s:s + len(props)] = e
        nsteps[s:s + len(props)] = st
        del props
    return states, energies, nsteps


def well_frame(prm):
    """Centre and inverse width of the harmonic approximation of the Morse well:
    xi = (r - re) * s with s = (m omega)^(1/2), omega = a (2 D / m)^(1/2).  In xi the
    ground states of all parameter sets have nearly the same shape."""
    d, a, re, _, mass = [float(v) for v in prm]
    return re, math.sqrt(a * math.sqrt(2.0 * d * mass))


class RadialBasis:
    """Per l: the leading `modes` left singular vectors of the training radial functions,
    sampled in the well's scaled coordinate xi (well_frame) on a fixed grid, so that the
    basis describes the shape of a ground state rather than its position and width."""

    def __init__(self, states, params, g: Grid2D, modes=64, nxi=1024, xi_max=10.0, u=None):
        self.modes, self.g = modes, g
        self.xi = np.linspace(-xi_max, xi_max, nxi)
        if u is not None:  # a saved basis
            self.u = np.asarray(u, dtype=np.float64)
            return
        psil = np.stack([self.to_xi(g.to_l(s.astype(np.float64)), p) for s, p in zip(states, params)])
        self.u = np.empty((g.nth, nxi, modes))
        for l in range(g.nth):
            x = psil[:, :, l].T  # [nxi, count]
            evals, evecs = np.linalg.eigh(x @ x.T)
            self.u[l] = evecs[:, ::-1][:, :modes]

    def to_xi(self, psil, prm):  # [nr, nl] on the radial grid -> [nxi, nl] on the xi grid
        from scipy.interpolate import CubicSpline
        re, sc = well_frame(prm)
        r = re + self.xi / sc
        out = CubicSpline(self.g.r, psil, axis=0)(np.clip(r, self.g.r_min, self.g.r_max))
        out[(r < self.g.r_min) | (r > self.g.r_max)] = 0.0
        return out

    def from_xi(self, psixi, prm):  # [nxi, nl] -> [nr, nl]
        from scipy.interpolate import CubicSpline
        re, sc = well_frame(prm)
        xi = (self.g.r - re) * sc
        out = CubicSpline(self.xi, psixi, axis=0)(np.clip(xi, self.xi[0], self.xi[-1]))
        out[(xi < self.xi[0]) | (xi > self.xi[-1])] = 0.0
        return out

    def coefficients(self, state, prm):
        psil = self.to_xi(self.g.to_l(np.asarray(state, dtype=np.float64)), prm)
        return np.einsum("lxm,xl->lm", self.u, psil)

    def state(self, coef, prm):
        return self.g.to_theta(self.from_xi(np.einsum("lxm,lm->xl", self.u, coef), prm))


class LearnedStart:
    def __init__(self, basis: RadialBasis, hidden=(256, 256, 256), seed=0, features=False, scaling="channel"):
        self.basis = basis
        self.inputs = physics_features if features else scale_params
        self.scaling = scaling
        nout = basis.g.nth * basis.modes
        self.net = so.Mlp([5, *hidden, nout], seed=seed)
        self.mean = None
        self.std = None

    def fit(self, params, states, steps=3000, lr=1e-3, lr_end=None, segments=10):
        """Full-batch Adam; with lr_end the rate falls geometrically from lr to lr_end
        over `segments` equal parts (the optimiser's moments carry across them)."""
        coef = np.stack([self.basis.coefficients(s, p).ravel() for s, p in zip(states, params)])
        self.mean = coef.mean(axis=0)
        if self.scaling == "channel":
            # one scale per l channel (the RMS spread of its modes): within a channel the
            # modes keep their physical weights, so the loss does not inflate modes that only
            # carry rounding noise of the training states
            sd = coef.std(axis=0).reshape(self.basis.g.nth, self.basis.modes)
            self.std = np.repeat(np.sqrt(np.mean(sd ** 2, axis=1)), self.basis.modes)
        else:
            self.std = coef.std(axis=0)
        self.std = self.std + 1e-12 * np.abs(coef).max()
        y = ((coef - self.mean) / self.std).astype(np.float32)
        x = self.inputs(params)
        if lr_end is None or segments <= 1:
            return self.net.train(x, y, steps=steps, lr=lr)
        per = max(1, steps // segments)
        rates = lr * (lr_end / lr) ** (np.arange(segments) / (segments - 1))
        return np.concatenate([self.net.train(x, y, steps=per, lr=float(r)) for r in rates])

    def standardized(self, params, states):
        """Network output and target, both standardized, for held-out checks."""
        coef = np.stack([self.basis.coefficients(s, p).ravel() for s, p in zip(states, params)])
        return self.net.forward(self.inputs(params)).astype(np.float64), (coef - self.mean) / self.std

    def predict(self, params):
        y = self.net.forward(self.inputs(params)).astype(np.float64)
        coef = y * self.std + self.mean
        return [self.basis.state(c.reshape(self.basis.g.nth, self.basis.modes), p) for c, p in zip(coef, params)]

    def save(self, path):
        """The trained network (FP32 master parameters), its target scaling and the radial
        basis (float32), with the grid they belong to, as one .npz file."""
        g, b = self.basis.g, self.basis
        np.savez_compressed(path, params=self.net.get_params(), widths=np.array(self.net.widths),
                            mean=self.mean, std=self.std, u=b.u.astype(np.float32), xi=b.xi,
                            grid=np.array([g.nr, g.nth, g.r_min, g.r_max]), modes=b.modes,
                            features=int(self.inputs is physics_features), scaling=self.scaling)

    @staticmethod
    def load(path):
        z = np.load(path, allow_pickle=False)
        nr, nth, r_min, r_max = z["grid"]
        g = Grid2D(int(nr), int(nth), float(r_min), float(r_max))
        xi = z["xi"]
        basis = RadialBasis(None, None, g, modes=int(z["modes"]), nxi=len(xi), xi_max=float(xi[-1]), u=z["u"])
        widths = [int(w) for w in z["widths"]]
        model = LearnedStart(basis, hidden=tuple(widths[1:-1]), features=bool(int(z["features"])),
                             scaling=str(z["scaling"]))
        model.net.set_params(z["params"])
        model.mean, model.std = z["mean"], z["std"]
        return model


def evaluate(model: LearnedStart, params, g: Grid2D, every=5, max_steps=20000, tol=1e-10, diagnose=False):
    """Held-out comparison: plain solver energies E* first, then both starts to |E - E*| <= 1e-8.
    diagnose: also relax from the held-out ground states projected on the radial basis (the
    best start the basis can represent) to separate basis truncation from network error."""
    true_states, e_star, steps_plain_full = ground_states(params, g, tol=tol, every=20, max_steps=max_steps)
    gauss = [problem(p, g) for p in params]
    _, steps_g, wall_g = relax(gauss, every=every, max_steps=max_steps, target=e_star)
    t0 = time.perf_counter()
    starts = model.predict(params)
    t_predict = time.perf_counter() - t0
    learned = [problem(p, g, psi0=s) for p, s in zip(params, starts)]
    _, steps_l, wall_l = relax(learned, every=every, max_steps=max_steps, target=e_star)
    wall_l += t_predict  # the network's forward pass and the basis sum are part of the learned start
    extra = {}
    if diagnose:
        proj = [model.basis.state(model.basis.coefficients(t, p), p) for t, p in zip(true_states, params)]
        _, steps_p, wall_p = relax([problem(p, g, psi0=s) for p, s in zip(params, proj)], every=every,
                                   max_steps=max_steps, target=e_star)
        err = [np.linalg.norm(s - t) / np.linalg.norm(t) for s, t in zip(starts, true_states)]
        perr = [np.linalg.norm(s - t) / np.linalg.norm(t) for s, t in zip(proj, true_states)]
        yh, th = model.standardized(params, true_states)
        # the isotropic (l = 0) and the anisotropic (l >= 1) parts of the start's error
        g = model.basis.g
        iso = [np.linalg.norm(g.to_l(s - t)[:, 0]) / np.linalg.norm(t) for s, t in zip(starts, true_states)]
        ani = [np.linalg.norm(g.to_l(s - t)[:, 1:]) / np.linalg.norm(t) for s, t in zip(starts, true_states)]
        extra = {"steps_projection_mean": float(np.mean(steps_p)), "wall_s_projection": wall_p,
                 "start_rel_l2_learned_median": float(np.median(err)),
                 "start_rel_l2_projection_median": float(np.median(perr)),
                 "start_rel_l2_l0_median": float(np.median(iso)), "start_rel_l2_l_ge_1_median": float(np.median(ani)),
                 "heldout_loss": float(np.mean((yh - th) ** 2))}
    return {**extra, "heldout": len(params), "energy_star_mean": float(np.mean(e_star)),
            "steps_gaussian_mean": float(np.mean(steps_g)), "steps_learned_mean": float(np.mean(steps_l)),
            "wall_s_gaussian": wall_g, "wall_s_learned": wall_l, "predict_s": t_predict,
            "wall_ratio_learned_over_gaussian": wall_l / wall_g,
            "steps_ratio_learned_over_gaussian": float(np.mean(steps_l) / np.mean(steps_g)),
            "converged_gaussian": int(np.sum(steps_g < max_steps)), "converged_learned": int(np.sum(steps_l < max_steps))}


# the network and basis trained at the full configuration (4096 ground states on the 2048 x 64
# grid, 64 radial modes per l), as written by `--model-out`
MODEL_2048x64 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "learned_start_2048x64.npz")


def time_to_ground_state(model_path=MODEL_2048x64, count=16, first=0, every=5, max_steps=20000):
    """Time to the ground state on `count` held-out parameter sets (default_rng(6), the sets
    first .. first + count - 1): the plain FP64 solver's converged energy E* first, then the
    plain Gaussian start and the learned start, each relaxed until |E - E*| <= 1e-8.  Wall
    times of both starts (the learned one including the network and the basis sum)."""
    model = LearnedStart.load(model_path)
    g = model.basis.g
    params = param_sets(256, 6)[first:first + count]
    t0 = time.perf_counter()
    _, e_star, _ = ground_states(params, g, tol=1e-10, every=20, max_steps=max_steps)
    t_star = time.perf_counter() - t0
    _, steps_g, wall_g = relax([problem(p, g) for p in params], every=every, max_steps=max_steps, target=e_star)
    t0 = time.perf_counter()
    starts = model.predict(params)
    t_predict = time.perf_counter() - t0
    _, steps_l, wall_l = relax([problem(p, g, psi0=s) for p, s in zip(params, starts)], every=every,
                               max_steps=max_steps, target=e_star)
    wall_l += t_predict
    return {"heldout_sets": [first, first + count], "grid": [g.nr, g.nth], "tolerance": 1e-8,
            "criterion": "E* of the plain FP64 imaginary-time solver run to |dE| <= 1e-10", "e_star_s": t_star,
            "wall_s_gaussian": wall_g, "wall_s_learned": wall_l, "predict_s": t_predict,
            "wall_ratio_learned_over_gaussian": wall_l / wall_g,
            "steps_gaussian_mean": float(np.mean(steps_g)), "steps_learned_mean": float(np.mean(steps_l)),
            "converged": [int(np.sum(steps_g < max_steps)), int(np.sum(steps_l < max_steps))]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--heldout", type=int, default=256)
    ap.add_argument("--nr", type=int, default=2048)
    ap.add_argument("--nth", type=int, default=64)
    ap.add_argument("--modes", type=int, default=64)
    ap.add_argument("--nxi", type=int, default=1024, help="points of the basis's scaled radial grid")
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-end", type=float, default=None)
    ap.add_argument("--diagnose", action="store_true")
    ap.add_argument("--features", action="store_true", help="physics features as the network's inputs")
    ap.add_argument("--scaling", default="channel", choices=["channel", "coef"],
                    help="standardise the targets per l channel or per coefficient")
    ap.add_argument("--out", default="learned_start.json")
    ap.add_argument("--model-out", default=None, help="write the trained model (.npz)")
    a = ap.parse_args()
    g = Grid2D(a.nr, a.nth)
    t0 = time.perf_counter()
    ptrain = param_sets(a.train, 5)
    states, energies, nsteps = ground_states(ptrain, g, progress=True)
    t_data = time.perf_counter() - t0
    print(f"training data: {t_data:.0f} s", flush=True)
    basis = RadialBasis(states, ptrain, g, a.modes, nxi=a.nxi)
    model = LearnedStart(basis, features=a.features, scaling=a.scaling)
    t0 = time.perf_counter()
    losses = model.fit(ptrain, states, steps=a.epochs, lr=a.lr, lr_end=a.lr_end)
    t_fit = time.perf_counter() - t0
    print(f"fit: {t_fit:.0f} s, loss {losses[0]:.3e} -> {losses[-1]:.3e}", flush=True)
    if a.model_out:
        model.save(a.model_out)
    res = evaluate(model, param_sets(a.heldout, 6), g, diagnose=a.diagnose)
    res.update({"train": a.train, "grid": [a.nr, a.nth], "modes": a.modes, "nxi": a.nxi,
                "train_loss_first": float(losses[0]),
                "train_loss_last": float(losses[-1]), "data_generation_s": t_data, "fit_s": t_fit,
                "epochs": a.epochs, "lr": a.lr, "lr_end": a.lr_end, "features": a.features, "scaling": a.scaling,
                "train_steps_mean": float(np.mean(nsteps))})
    with open(a.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
