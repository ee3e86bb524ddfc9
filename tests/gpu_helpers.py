"""Shared helpers for the GPU parity tests (imports the oracle as the checker)."""
import numpy as np

from numpyro_gb300 import datasets, models
from oracle import potentials_ref as PR


def family_cases(small=True):
    """(name, registry model, oracle potential_and_grad) for each family at test sizes."""
    out = []
    y, s = datasets.eight_schools(0)
    out.append(("hier_nc", models.HierarchicalNormal(y, s), PR.make_potential("hier_nc", y.astype(np.float64),
                                                                                s.astype(np.float64))))
    X, yy, _ = datasets.covtype_like(seed=1, n=3000 if small else 581012, n_cont=4, n_bin=6)
    out.append(("logreg", models.LogisticRegression(X, yy), PR.make_potential("logreg", X.astype(np.float64),
                                                                              yy.astype(np.float64))))
    Xh, yh, _ = datasets.horseshoe_data(seed=2, n=200, p=50, nonzero=5)
    out.append(("horseshoe", models.HorseshoeRegression(Xh, yh),
                PR.make_potential("horseshoe", Xh.astype(np.float64), yh.astype(np.float64))))
    out.append(("horseshoe_nc", models.HorseshoeRegression(Xh, yh, noncentered=True),
                PR.make_potential("horseshoe_nc", Xh.astype(np.float64), yh.astype(np.float64))))
    r, _ = datasets.sv_returns(seed=3, T=300)
    out.append(("sv", models.StochasticVolatility(r), PR.make_potential("sv", r.astype(np.float64))))
    r2, _ = datasets.sv_returns(seed=4, T=1000)
    out.append(("sv_nc", models.StochasticVolatility(r2, noncentered=True),
                PR.make_potential("sv_nc", r2.astype(np.float64))))
    return out


def typical_points(name, model, rng, C):
    """Latent points in a plausible region of each posterior."""
    D = model.latent_dim
    if name == "sv":
        T = D - 2
        z = np.empty((C, D))
        z[:, :T] = np.log(0.01) + 0.3 * rng.standard_normal((C, T))
        z[:, T] = np.log(8.0) + 0.3 * rng.standard_normal(C)
        z[:, T + 1] = np.log(0.02) + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    if name == "sv_nc":
        T = D - 2
        z = np.empty((C, D))
        z[:, :T] = 0.3 * rng.standard_normal((C, T))
        z[:, T] = np.log(8.0) + 0.3 * rng.standard_normal(C)
        z[:, T + 1] = np.log(0.05) + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    if name == "logreg":
        return (0.3 * rng.standard_normal((C, D))).astype(np.float32)
    if name == "horseshoe_nc":
        P = (D - 2) // 2
        z = np.empty((C, D))
        z[:, :P] = rng.standard_normal((C, P))
        z[:, P] = 0.3 * rng.standard_normal(C)
        z[:, P + 1] = -2.0 + 0.3 * rng.standard_normal(C)
        z[:, P + 2:] = rng.standard_normal((C, P))
        return z.astype(np.float32)
    if name == "horseshoe":
        P = (D - 2) // 2
        z = np.empty((C, D))
        z[:, :P] = 0.1 * rng.standard_normal((C, P))
        z[:, P:2 * P] = rng.standard_normal((C, P))
        z[:, 2 * P] = 0.3 * rng.standard_normal(C)
        z[:, 2 * P + 1] = -2.0 + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    return rng.uniform(-2, 2, (C, D)).astype(np.float32)


def replay_parity(kernel, state, cmodel, seed, transitions, max_tree_depth=10, threads=0, fp32_oracle=False):
    """Runs ``transitions`` GPU transitions of ``kernel`` from ``state`` (after warmup, so
    without adaptation) and replays each one with the FP64 C oracle from the GPU's own
    starting state (position, step size, mass rows) at the same Philox stream addresses.
    Returns counts of identical tree sizes / divergence flags and the relative position
    errors of the transitions whose tree sizes agree.  With ``fp32_oracle`` the FP32 build of
    the same C restatement (numpyro's algorithm in its float32 dtype) is replayed from the
    same states too, and its agreement with FP64 is counted as ``same32``: how far float32
    rounding alone moves the tree decisions of this model."""
    from oracle import build_oracle as B

    lib = B.load("f64")
    lib32 = B.load("f32") if fp32_oracle else None
    same, same32, total, zerr, aperr, zerr32, aperr32, st = 0, 0, 0, [], [], [], [], state
    for _ in range(transitions):
        z0 = st.z.cpu().numpy()
        step = st.adapt_state.step_size.cpu().numpy()
        inv = st.adapt_state.inverse_mass_matrix.cpu().numpy()
        msq = st.adapt_state.mass_matrix_sqrt.cpu().numpy()
        key = st.rng_key.cpu().numpy().astype(np.uint32)
        new = kernel.sample(st)
        ns = new.num_steps.cpu().numpy()
        dv = new.diverging.cpu().numpy().astype(bool)
        zg = new.z.cpu().numpy()
        ap = new.accept_prob.cpu().numpy()
        ref = B.transitions(lib, cmodel, z0, step, inv, msq, key[:, 0], key[:, 1], seed,
                            max_tree_depth=max_tree_depth, threads=threads)
        if lib32 is not None:
            r32 = B.transitions(lib32, cmodel, z0, step, inv, msq, key[:, 0], key[:, 1], seed,
                                max_tree_depth=max_tree_depth, threads=threads)
            agree32 = (r32["num_steps"] == ref["num_steps"]) & (r32["diverging"] == ref["diverging"])
            same32 += int(np.sum(agree32))
            for c in np.nonzero(agree32)[0]:
                rz = ref["z"][c].astype(np.float64)
                zerr32.append(np.max(np.abs(rz - r32["z"][c]) / (np.abs(rz) + 1e-2)))
                aperr32.append(abs(ref["accept_prob"][c] - r32["accept_prob"][c]))
        for c in range(z0.shape[0]):
            total += 1
            if ref["num_steps"][c] == ns[c] and ref["diverging"][c] == dv[c]:
                same += 1
                aperr.append(abs(ref["accept_prob"][c] - ap[c]))
                rz = ref["z"][c].astype(np.float64)
                zerr.append(np.max(np.abs(rz - zg[c]) / (np.abs(rz) + 1e-2)))
        st = new
    return {"same": same, "total": total, "frac": same / total, "zerr": np.array(zerr), "aperr": np.array(aperr),
            "state": st, "same32": same32 if lib32 is not None else None, "zerr32": np.array(zerr32),
            "aperr32": np.array(aperr32)}


def cmodel_of(model, chains_per_model=1):
    """The C oracle's copy of a registry model (oracle/nuts_ref.c nutsref_model)."""
    from oracle import build_oracle as B

    return B.model_from_registry(model, chains_per_model)
