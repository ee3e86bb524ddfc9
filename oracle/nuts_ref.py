"""FP64 restatement of numpyro's HMC/NUTS (oracle side, test infrastructure).

Eager Python control flow in the style of numpyro's
``control_flow_prims_disabled`` (numpyro/util.py:126-173); every function
follows the reference function named in its docstring.  Randomness is not
JAX's threefry: it is drawn from the Philox stream of ``oracle/philox.py`` at
addresses (chain, transition, purpose, index, sub), the same addresses the
CUDA engine uses, so the oracle and the GPU see identical bits.
"""
from collections import namedtuple
import math

import numpy as np

from . import philox

# numpyro/infer/hmc_util.py:16-56
AdaptWindow = namedtuple("AdaptWindow", ["start", "end"])
HMCAdaptState = namedtuple(
    "HMCAdaptState",
    ["step_size", "inverse_mass_matrix", "mass_matrix_sqrt", "mass_matrix_sqrt_inv",
     "ss_state", "mm_state", "window_idx", "rng_key"],
)
IntegratorState = namedtuple("IntegratorState", ["z", "r", "potential_energy", "z_grad"])
TreeInfo = namedtuple(
    "TreeInfo",
    ["z_left", "r_left", "z_left_grad", "z_right", "r_right", "z_right_grad",
     "z_proposal", "z_proposal_pe", "z_proposal_grad", "z_proposal_energy",
     "depth", "weight", "r_sum", "turning", "diverging", "sum_accept_probs", "num_proposals"],
)
# numpyro/infer/hmc.py:31-47
HMCState = namedtuple(
    "HMCState",
    ["i", "z", "z_grad", "potential_energy", "energy", "r", "trajectory_length",
     "num_steps", "accept_prob", "mean_accept_prob", "diverging", "adapt_state", "rng_key"],
)
# rng_key of the oracle: (seed, chain, transition counter n)
RngKey = namedtuple("RngKey", ["seed", "chain", "n"])

FLOAT64_TINY = np.finfo(np.float64).tiny
FLOAT64_MAX = np.finfo(np.float64).max


def _sigmoid(x):
    if x >= 0:
        return 1.0 / (1.0 + math.exp(-x))
    e = math.exp(x)
    return e / (1.0 + e)


def _logaddexp(a, b):
    return float(np.logaddexp(a, b))


# ----------------------------------------------------------------------------
# dual averaging / Welford / schedule
# ----------------------------------------------------------------------------
def dual_averaging(t0=10, kappa=0.75, gamma=0.05):
    """hmc_util.py:60-130."""

    def init_fn(prox_center=0.0):
        return (0.0, 0.0, 0.0, 0, prox_center)

    def update_fn(g, state):
        x_t, x_avg, g_avg, t, prox_center = state
        t = t + 1
        g_avg = (1 - 1 / (t + t0)) * g_avg + g / (t + t0)
        x_t = prox_center - (t ** 0.5) / gamma * g_avg
        weight_t = t ** (-kappa)
        x_avg = (1 - weight_t) * x_avg + weight_t * x_t
        return (x_t, x_avg, g_avg, t, prox_center)

    return init_fn, update_fn


def welford_covariance(diagonal=True):
    """hmc_util.py:133-239 (diagonal and dense)."""

    def init_fn(size):
        shape = (size,) if diagonal else (size, size)
        return (np.zeros(size), np.zeros(shape), 0)

    def update_fn(sample, state):
        mean, m2, n = state
        n = n + 1
        delta_pre = sample - mean
        mean = mean + delta_pre / n
        delta_post = sample - mean
        if m2.ndim == 1:
            m2 = m2 + delta_pre * delta_post
        else:
            m2 = m2 + np.outer(delta_post, delta_pre)
        return (mean, m2, n)

    def final_fn(state, regularize=False):
        mean, m2, n = state
        cov = m2 / (n - 1)
        if regularize:
            scaled_cov = (n / (n + 5)) * cov
            shrinkage = 1e-3 * (5 / (n + 5))
            if scaled_cov.ndim == 1:
                cov = scaled_cov + shrinkage
            else:
                cov = scaled_cov + shrinkage * np.identity(mean.shape[0])
        if cov.ndim == 2:
            tril_inv = np.swapaxes(np.linalg.cholesky(cov[::-1, ::-1])[::-1, ::-1], -2, -1)
            cov_inv_sqrt = np.linalg.solve(np.tril(tril_inv), np.identity(cov.shape[-1]))
        else:
            tril_inv = np.sqrt(cov)
            cov_inv_sqrt = np.reciprocal(tril_inv)
        return cov, cov_inv_sqrt, tril_inv

    return init_fn, update_fn, final_fn


def build_adaptation_schedule(num_steps):
    """hmc_util.py:387-436 (Stan windows)."""
    adaptation_schedule = []
    if num_steps < 20:
        adaptation_schedule.append(AdaptWindow(0, num_steps - 1))
        return adaptation_schedule
    start_buffer_size = 75
    end_buffer_size = 50
    init_window_size = 25
    if (start_buffer_size + end_buffer_size + init_window_size) > num_steps:
        start_buffer_size = int(0.15 * num_steps)
        end_buffer_size = int(0.1 * num_steps)
        init_window_size = num_steps - start_buffer_size - end_buffer_size
    adaptation_schedule.append(AdaptWindow(start=0, end=start_buffer_size - 1))
    end_window_start = num_steps - end_buffer_size
    next_window_size = init_window_size
    next_window_start = start_buffer_size
    while next_window_start < end_window_start:
        cur_window_start, cur_window_size = next_window_start, next_window_size
        if 3 * cur_window_size <= end_window_start - cur_window_start:
            next_window_size = 2 * cur_window_size
        else:
            cur_window_size = end_window_start - cur_window_start
        next_window_start = cur_window_start + cur_window_size
        adaptation_schedule.append(AdaptWindow(cur_window_start, next_window_start - 1))
    adaptation_schedule.append(AdaptWindow(end_window_start, num_steps - 1))
    return adaptation_schedule


# ----------------------------------------------------------------------------
# kinetic energy and integrator
# ----------------------------------------------------------------------------
def euclidean_kinetic_energy(inverse_mass_matrix, r):
    """hmc_util.py:1183-1200."""
    r = np.asarray(r, np.float64)
    m = np.asarray(inverse_mass_matrix, np.float64)
    v = m @ r if m.ndim == 2 else m * r
    return 0.5 * float(np.dot(v, r))


def kinetic_grad(inverse_mass_matrix, r):
    """hmc_util.py:1203-1223."""
    m = np.asarray(inverse_mass_matrix, np.float64)
    return m @ r if m.ndim == 2 else m * r


def velocity_verlet(potential_and_grad, kinetic_fn=euclidean_kinetic_energy):
    """hmc_util.py:262-311.  ``potential_and_grad(z) -> (pe, grad)``."""

    def init_fn(z, r, potential_energy=None, z_grad=None):
        if potential_energy is None or z_grad is None:
            potential_energy, z_grad = potential_and_grad(z)
        return IntegratorState(z, r, potential_energy, z_grad)

    def update_fn(step_size, inverse_mass_matrix, state):
        z, r, _, z_grad = state
        r = r - 0.5 * step_size * z_grad
        r_grad = kinetic_grad(inverse_mass_matrix, r)
        z = z + step_size * r_grad
        potential_energy, z_grad = potential_and_grad(z)
        r = r - 0.5 * step_size * z_grad
        return IntegratorState(z, r, potential_energy, z_grad)

    return init_fn, update_fn


# ----------------------------------------------------------------------------
# NUTS tree
# ----------------------------------------------------------------------------
def momentum_angle(inverse_mass_matrix, r_left, r_right, r_sum):
    """hmc_util.py:710-737 (dynamic termination, Betancourt A.4.2)."""
    v_left = kinetic_grad(inverse_mass_matrix, r_left)
    v_right = kinetic_grad(inverse_mass_matrix, r_right)
    r_sum = r_sum - (r_left + r_right) / 2
    return float(np.dot(v_left, r_sum)), float(np.dot(v_right, r_sum))


def is_turning(inverse_mass_matrix, r_left, r_right, r_sum):
    """hmc_util.py:740-746."""
    left, right = momentum_angle(inverse_mass_matrix, np.atleast_1d(r_left),
                                 np.atleast_1d(r_right), np.atleast_1d(r_sum))
    return (left <= 0) or (right <= 0)


def leaf_idx_to_ckpt_idxs(n):
    """hmc_util.py:941-958."""
    idx_max = bin(n >> 1).count("1")
    num_subtrees = bin((~n & (n + 1)) - 1).count("1")
    idx_min = idx_max - num_subtrees + 1
    return idx_min, idx_max


def is_iterative_turning(inverse_mass_matrix, r, r_sum, r_ckpts, r_sum_ckpts, idx_min, idx_max):
    """hmc_util.py:961-981."""
    i = idx_max
    turning = False
    while i >= idx_min and not turning:
        subtree_r_sum = r_sum - r_sum_ckpts[i] + r_ckpts[i]
        turning = is_turning(inverse_mass_matrix, r_ckpts[i], r, subtree_r_sum)
        i -= 1
    return turning


def _uniform_transition_kernel(current_tree, new_tree):
    """hmc_util.py:749-753."""
    return _sigmoid(new_tree.weight - current_tree.weight)


def _biased_transition_kernel(current_tree, new_tree):
    """hmc_util.py:756-764."""
    if new_tree.turning or new_tree.diverging:
        return 0.0
    return min(math.exp(min(new_tree.weight - current_tree.weight, 700.0)), 1.0)


def _combine_tree(current_tree, new_tree, inverse_mass_matrix, going_right, u, biased_transition):
    """hmc_util.py:767-848.  ``u`` is the injected uniform of the Bernoulli."""
    if going_right:
        z_left, r_left, z_left_grad = current_tree.z_left, current_tree.r_left, current_tree.z_left_grad
        z_right, r_right, z_right_grad = new_tree.z_right, new_tree.r_right, new_tree.z_right_grad
    else:
        z_left, r_left, z_left_grad = new_tree.z_left, new_tree.r_left, new_tree.z_left_grad
        z_right, r_right, z_right_grad = current_tree.z_right, current_tree.r_right, current_tree.z_right_grad
    r_sum = current_tree.r_sum + new_tree.r_sum
    if biased_transition:
        transition_prob = _biased_transition_kernel(current_tree, new_tree)
        turning = new_tree.turning or is_turning(inverse_mass_matrix, r_left, r_right, r_sum)
    else:
        transition_prob = _uniform_transition_kernel(current_tree, new_tree)
        turning = current_tree.turning
    transition = u < transition_prob
    src = new_tree if transition else current_tree
    return TreeInfo(
        z_left, r_left, z_left_grad, z_right, r_right, z_right_grad,
        src.z_proposal, src.z_proposal_pe, src.z_proposal_grad, src.z_proposal_energy,
        current_tree.depth + 1,
        _logaddexp(current_tree.weight, new_tree.weight),
        r_sum, turning, new_tree.diverging,
        current_tree.sum_accept_probs + new_tree.sum_accept_probs,
        current_tree.num_proposals + new_tree.num_proposals,
    )


def _build_basetree(vv_update, kinetic_fn, z, r, z_grad, inverse_mass_matrix, step_size,
                    going_right, energy_current, max_delta_energy):
    """hmc_util.py:851-894."""
    step_size = step_size if going_right else -step_size
    z_new, r_new, pe_new, z_new_grad = vv_update(step_size, inverse_mass_matrix, (z, r, energy_current, z_grad))
    energy_new = pe_new + kinetic_fn(inverse_mass_matrix, r_new)
    delta_energy = energy_new - energy_current
    if math.isnan(delta_energy):
        delta_energy = math.inf
    tree_weight = -delta_energy
    diverging = delta_energy > max_delta_energy
    accept_prob = min(math.exp(min(-delta_energy, 700.0)), 1.0)
    return TreeInfo(z_new, r_new, z_new_grad, z_new, r_new, z_new_grad,
                    z_new, pe_new, z_new_grad, energy_new,
                    0, tree_weight, r_new, False, diverging, accept_prob, 1)


def _get_leaf(tree, going_right):
    """hmc_util.py:897-904."""
    if going_right:
        return tree.z_right, tree.r_right, tree.z_right_grad
    return tree.z_left, tree.r_left, tree.z_left_grad


def _iterative_build_subtree(prototype_tree, vv_update, kinetic_fn, inverse_mass_matrix, step_size,
                             going_right, rng, energy_current, max_delta_energy, r_ckpts, r_sum_ckpts):
    """hmc_util.py:984-1085.  ``rng(j)`` returns the uniform for leaf j >= 1."""
    max_num_proposals = 2 ** prototype_tree.depth
    r_ckpts = r_ckpts.copy()
    r_sum_ckpts = r_sum_ckpts.copy()
    current_tree = prototype_tree._replace(num_proposals=0)
    turning = False
    while (current_tree.num_proposals < max_num_proposals) and not turning and not current_tree.diverging:
        z, r, z_grad = _get_leaf(current_tree, going_right)
        new_leaf = _build_basetree(vv_update, kinetic_fn, z, r, z_grad, inverse_mass_matrix, step_size,
                                   going_right, energy_current, max_delta_energy)
        leaf_idx = current_tree.num_proposals
        if leaf_idx == 0:
            new_tree = new_leaf
        else:
            new_tree = _combine_tree(current_tree, new_leaf, inverse_mass_matrix, going_right,
                                     rng(leaf_idx), False)
        ckpt_idx_min, ckpt_idx_max = leaf_idx_to_ckpt_idxs(leaf_idx)
        r = new_leaf.r_right
        r_sum = new_tree.r_sum
        if leaf_idx % 2 == 0:
            r_ckpts[ckpt_idx_max] = r
            r_sum_ckpts[ckpt_idx_max] = r_sum
        turning = is_iterative_turning(inverse_mass_matrix, r, r_sum, r_ckpts, r_sum_ckpts,
                                       ckpt_idx_min, ckpt_idx_max)
        current_tree = new_tree
    tree = current_tree
    return TreeInfo(tree.z_left, tree.r_left, tree.z_left_grad, tree.z_right, tree.r_right, tree.z_right_grad,
                    tree.z_proposal, tree.z_proposal_pe, tree.z_proposal_grad, tree.z_proposal_energy,
                    prototype_tree.depth, tree.weight, tree.r_sum, turning, tree.diverging,
                    tree.sum_accept_probs, tree.num_proposals)


def build_tree(verlet_update, kinetic_fn, verlet_state, inverse_mass_matrix, step_size, rng_key,
               max_delta_energy=1000.0, max_tree_depth=10):
    """hmc_util.py:1088-1180 with the Philox stream of (seed, chain, n)."""
    if isinstance(max_tree_depth, tuple):
        max_tree_depth_current, max_tree_depth = max_tree_depth
    else:
        max_tree_depth_current = max_tree_depth
    z, r, potential_energy, z_grad = verlet_state
    energy_current = potential_energy + kinetic_fn(inverse_mass_matrix, r)
    latent_size = np.size(r)
    r_ckpts = np.zeros((max_tree_depth, latent_size))
    r_sum_ckpts = np.zeros((max_tree_depth, latent_size))
    tree = TreeInfo(z, r, z_grad, z, r, z_grad, z, potential_energy, z_grad, energy_current,
                    0, 0.0, r, False, False, 0.0, 0)
    seed, chain, n = rng_key
    while tree.depth < max_tree_depth_current and not tree.turning and not tree.diverging:
        words = philox.words_to_uniform(philox.draw(seed, chain, n, philox.DOUBLING, tree.depth))
        going_right = bool(words[0] < 0.5)
        depth = tree.depth

        def leaf_rng(j, depth=depth):
            return philox.uniform(seed, chain, n, philox.LEAF, depth, j)

        new_tree = _iterative_build_subtree(tree, verlet_update, kinetic_fn, inverse_mass_matrix, step_size,
                                            going_right, leaf_rng, energy_current, max_delta_energy,
                                            r_ckpts, r_sum_ckpts)
        tree = _combine_tree(tree, new_tree, inverse_mass_matrix, going_right, float(words[1]), True)
    return tree


# ----------------------------------------------------------------------------
# adaptation
# ----------------------------------------------------------------------------
def momentum_generator(mass_matrix_sqrt, rng_key, purpose=philox.MOMENTUM, sub=0):
    """hmc.py:92-110 with Philox normals at (chain, n, purpose)."""
    seed, chain, n = rng_key
    m = np.asarray(mass_matrix_sqrt, np.float64)
    eps = philox.normals(seed, chain, n, purpose, m.shape[0], sub)
    return m @ eps if m.ndim == 2 else m * eps


def find_reasonable_step_size(potential_and_grad, kinetic_fn, init_step_size, inverse_mass_matrix,
                              z_info, rng_key, momentum_fn=None):
    """hmc_util.py:314-384.  Trial t draws its momentum at HEURISTIC sub=t.

    As in the reference (hmc_util.py:356) the momentum generator is handed the
    inverse mass matrix."""
    target_accept_prob = math.log(0.8)
    _, vv_update = velocity_verlet(potential_and_grad, kinetic_fn)
    z, _, potential_energy, z_grad = z_info
    if potential_energy is None or z_grad is None:
        potential_energy, z_grad = potential_and_grad(z)
    step_size, last_direction, direction, trial = init_step_size, 0, 0, 0

    def cond(step_size, last_direction, direction):
        not_small = (step_size > FLOAT64_TINY) or (direction >= 0)
        not_large = (step_size < FLOAT64_MAX) or (direction <= 0)
        return not_small and not_large and ((last_direction == 0) or (direction == last_direction))

    while cond(step_size, last_direction, direction):
        step_size = (2.0 ** direction) * step_size
        if momentum_fn is not None:
            r = momentum_fn(inverse_mass_matrix)
        else:
            r = momentum_generator(inverse_mass_matrix, rng_key, philox.HEURISTIC, trial)
        _, r_new, pe_new, _ = vv_update(step_size, inverse_mass_matrix, (z, r, potential_energy, z_grad))
        energy_current = kinetic_fn(inverse_mass_matrix, r) + potential_energy
        energy_new = kinetic_fn(inverse_mass_matrix, r_new) + pe_new
        delta_energy = energy_new - energy_current
        direction_new = 1 if target_accept_prob < -delta_energy else -1
        last_direction, direction = direction, direction_new
        trial += 1
    return step_size


def _initialize_mass_matrix(size, inverse_mass_matrix, dense_mass):
    """hmc_util.py:439-515 (unstructured case)."""
    if inverse_mass_matrix is None:
        inverse_mass_matrix = np.identity(size) if dense_mass else np.ones(size)
        return inverse_mass_matrix, inverse_mass_matrix, inverse_mass_matrix
    inverse_mass_matrix = np.asarray(inverse_mass_matrix, np.float64)
    if dense_mass:
        if inverse_mass_matrix.ndim == 1:
            inverse_mass_matrix = np.diag(inverse_mass_matrix)
        sqrt_inv = np.swapaxes(np.linalg.cholesky(inverse_mass_matrix[::-1, ::-1])[::-1, ::-1], -2, -1)
        mm_sqrt = np.linalg.solve(np.tril(sqrt_inv), np.identity(size))
        return inverse_mass_matrix, mm_sqrt, sqrt_inv
    if inverse_mass_matrix.ndim == 2:
        inverse_mass_matrix = np.diag(inverse_mass_matrix)
    sqrt_inv = np.sqrt(inverse_mass_matrix)
    return inverse_mass_matrix, np.reciprocal(sqrt_inv), sqrt_inv


def warmup_adapter(num_adapt_steps, find_reasonable_step_size=None, adapt_step_size=True,
                   adapt_mass_matrix=True, dense_mass=False, target_accept_prob=0.8,
                   regularize_mass_matrix=True):
    """hmc_util.py:518-707.  ``find_reasonable_step_size(step_size, inv_mass, z_info, rng_key)``."""
    if find_reasonable_step_size is None:
        find_reasonable_step_size = lambda step_size, *args: step_size  # noqa: E731
    ss_init, ss_update = dual_averaging()
    mm_init, mm_update, mm_final = welford_covariance(diagonal=not dense_mass)
    adaptation_schedule = build_adaptation_schedule(num_adapt_steps)
    num_windows = len(adaptation_schedule)

    def init_fn(z_info, rng_key, step_size=1.0, inverse_mass_matrix=None, mass_matrix_size=None):
        size = mass_matrix_size if mass_matrix_size is not None else np.size(z_info[0])
        inverse_mass_matrix, mm_sqrt, mm_sqrt_inv = _initialize_mass_matrix(size, inverse_mass_matrix, dense_mass)
        if adapt_step_size:
            step_size = find_reasonable_step_size(step_size, inverse_mass_matrix, z_info, rng_key)
        ss_state = ss_init(math.log(10 * step_size))
        mm_state = mm_init(inverse_mass_matrix.shape[-1])
        return HMCAdaptState(step_size, inverse_mass_matrix, mm_sqrt, mm_sqrt_inv, ss_state, mm_state, 0, rng_key)

    def _update_at_window_end(z_info, rng_key_ss, state):
        step_size, inverse_mass_matrix, mm_sqrt, mm_sqrt_inv, ss_state, mm_state, window_idx, rng_key = state
        if adapt_mass_matrix:
            inverse_mass_matrix, mm_sqrt, mm_sqrt_inv = mm_final(mm_state, regularize=regularize_mass_matrix)
            mm_state = mm_init(inverse_mass_matrix.shape[-1])
        if adapt_step_size:
            step_size = find_reasonable_step_size(step_size, inverse_mass_matrix, z_info, rng_key_ss)
            ss_state = ss_init(math.log(10) + math.log(step_size))
        return HMCAdaptState(step_size, inverse_mass_matrix, mm_sqrt, mm_sqrt_inv, ss_state, mm_state,
                             window_idx, rng_key)

    def update_fn(t, accept_prob, z_info, state):
        step_size, inverse_mass_matrix, mm_sqrt, mm_sqrt_inv, ss_state, mm_state, window_idx, rng_key = state
        if adapt_step_size:
            ss_state = ss_update(target_accept_prob - accept_prob, ss_state)
            log_step_size, log_step_size_avg = ss_state[0], ss_state[1]
            step_size = math.exp(log_step_size_avg) if t == (num_adapt_steps - 1) else math.exp(log_step_size)
            step_size = min(max(step_size, FLOAT64_TINY), FLOAT64_MAX)
        is_middle_window = (0 < window_idx) and (window_idx < (num_windows - 1))
        if adapt_mass_matrix and is_middle_window:
            mm_state = mm_update(np.asarray(z_info[0], np.float64), mm_state)
        t_at_window_end = t == adaptation_schedule[window_idx][1]
        if t_at_window_end:
            window_idx = window_idx + 1
        state = HMCAdaptState(step_size, inverse_mass_matrix, mm_sqrt, mm_sqrt_inv, ss_state, mm_state,
                              window_idx, rng_key)
        if t_at_window_end and is_middle_window:
            state = _update_at_window_end(z_info, (rng_key, t), state)
        return state

    return init_fn, update_fn


# ----------------------------------------------------------------------------
# hmc(): init_kernel / sample_kernel
# ----------------------------------------------------------------------------
def hmc(potential_and_grad, algo="NUTS", kinetic_fn=euclidean_kinetic_energy):
    """hmc.py:113-538 for one chain.  Returns (init_kernel, sample_kernel)."""
    cfg = {}

    def init_kernel(init_params, num_warmup, step_size=1.0, inverse_mass_matrix=None,
                    adapt_step_size=True, adapt_mass_matrix=True, dense_mass=False,
                    target_accept_prob=0.8, *, num_steps=None, trajectory_length=2 * math.pi,
                    max_tree_depth=10, find_heuristic_step_size=False, regularize_mass_matrix=True,
                    rng_key=None, max_delta_energy=1000.0):
        cfg["wa_steps"] = num_warmup
        cfg["max_treedepth"] = max_tree_depth if isinstance(max_tree_depth, tuple) else (max_tree_depth, max_tree_depth)
        cfg["fixed_num_steps"] = num_steps
        cfg["max_delta_energy"] = max_delta_energy
        seed, chain = rng_key
        z = np.asarray(init_params, np.float64)
        pe, z_grad = potential_and_grad(z)
        frs = None
        if find_heuristic_step_size:
            def frs(step_size, inv_mass, z_info, key):
                if isinstance(key, tuple) and len(key) == 2 and isinstance(key[0], RngKey):
                    k, t = key
                    key = RngKey(k.seed, k.chain, t)
                return find_reasonable_step_size(potential_and_grad, kinetic_fn, step_size, inv_mass, z_info, key)
        wa_init, wa_update = warmup_adapter(num_warmup, find_reasonable_step_size=frs,
                                            adapt_step_size=adapt_step_size, adapt_mass_matrix=adapt_mass_matrix,
                                            dense_mass=dense_mass, target_accept_prob=target_accept_prob,
                                            regularize_mass_matrix=regularize_mass_matrix)
        cfg["wa_update"] = wa_update
        key0 = RngKey(seed, chain, philox.INIT_TRANSITION)
        wa_state = wa_init(IntegratorState(z, None, pe, z_grad), key0, step_size,
                           inverse_mass_matrix=inverse_mass_matrix, mass_matrix_size=z.size)
        # numpyro draws an initial momentum (hmc.py:340) that NUTS never uses
        # (state.r is None); energy at init uses r = 0 here.
        energy = pe
        return HMCState(0, z, z_grad, pe, energy, None, trajectory_length, 0, 0.0, 0.0, False, wa_state,
                        RngKey(seed, chain, 0))

    def _hmc_next(step_size, inverse_mass_matrix, vv_state, rng_key, trajectory_length):
        """hmc.py:364-414."""
        _, vv_update = velocity_verlet(potential_and_grad, kinetic_fn)
        if cfg["fixed_num_steps"] is not None:
            num_steps = cfg["fixed_num_steps"]
        else:
            num_steps = int(math.ceil(trajectory_length / step_size))
        if trajectory_length is not None:
            step_size = trajectory_length / num_steps
        vv_state_new = vv_state
        for _ in range(num_steps):
            vv_state_new = vv_update(step_size, inverse_mass_matrix, vv_state_new)
        energy_old = vv_state.potential_energy + kinetic_fn(inverse_mass_matrix, vv_state.r)
        energy_new = vv_state_new.potential_energy + kinetic_fn(inverse_mass_matrix, vv_state_new.r)
        delta_energy = energy_new - energy_old
        if math.isnan(delta_energy):
            delta_energy = math.inf
        accept_prob = min(math.exp(min(-delta_energy, 700.0)), 1.0)
        diverging = delta_energy > cfg["max_delta_energy"]
        seed, chain, n = rng_key
        u = philox.uniform(seed, chain, n, philox.HMC_ACCEPT, 0)
        if u < accept_prob:
            return vv_state_new, energy_new, num_steps, accept_prob, diverging
        return vv_state, energy_old, num_steps, accept_prob, diverging

    def _nuts_next(step_size, inverse_mass_matrix, vv_state, rng_key, max_treedepth_current):
        """hmc.py:416-455."""
        _, vv_update = velocity_verlet(potential_and_grad, kinetic_fn)
        tree = build_tree(vv_update, kinetic_fn, vv_state, inverse_mass_matrix, step_size, rng_key,
                          max_delta_energy=cfg["max_delta_energy"],
                          max_tree_depth=(max_treedepth_current, max(cfg["max_treedepth"])))
        accept_prob = tree.sum_accept_probs / tree.num_proposals
        vv_state = IntegratorState(tree.z_proposal, vv_state.r, tree.z_proposal_pe, tree.z_proposal_grad)
        return vv_state, tree.z_proposal_energy, tree.num_proposals, accept_prob, tree.diverging

    def sample_kernel(hmc_state):
        """hmc.py:459-530."""
        seed, chain, n = hmc_state.rng_key
        key = RngKey(seed, chain, n)
        r = momentum_generator(hmc_state.adapt_state.mass_matrix_sqrt, key)
        vv_state = IntegratorState(hmc_state.z, r, hmc_state.potential_energy, hmc_state.z_grad)
        wa_steps = cfg["wa_steps"]
        if algo == "HMC":
            vv_state, energy, num_steps, accept_prob, diverging = _hmc_next(
                hmc_state.adapt_state.step_size, hmc_state.adapt_state.inverse_mass_matrix, vv_state, key,
                hmc_state.trajectory_length)
        else:
            mtd = cfg["max_treedepth"][0] if hmc_state.i < wa_steps else cfg["max_treedepth"][1]
            vv_state, energy, num_steps, accept_prob, diverging = _nuts_next(
                hmc_state.adapt_state.step_size, hmc_state.adapt_state.inverse_mass_matrix, vv_state, key, mtd)
        adapt_state = hmc_state.adapt_state
        if hmc_state.i < wa_steps:
            adapt_state = cfg["wa_update"](hmc_state.i, accept_prob, vv_state, adapt_state._replace(rng_key=key))
        itr = hmc_state.i + 1
        nn = itr if hmc_state.i < wa_steps else itr - wa_steps
        mean_accept_prob = hmc_state.mean_accept_prob + (accept_prob - hmc_state.mean_accept_prob) / nn
        return HMCState(itr, vv_state.z, vv_state.z_grad, vv_state.potential_energy, energy, None,
                        hmc_state.trajectory_length, num_steps, accept_prob, mean_accept_prob, diverging,
                        adapt_state, RngKey(seed, chain, n + 1))

    return init_kernel, sample_kernel


def init_to_uniform(seed, chain, dim, radius=2.0, attempt=0):
    """initialization.py:95 + infer/util.py:456-463: U(-radius, radius) per coordinate."""
    u = philox.uniforms_block(seed, chain, attempt, philox.INIT, dim)
    return -radius + 2.0 * radius * u


def run_chain(potential_and_grad, dim, seed, chain, num_warmup, num_samples, algo="NUTS",
              init_params=None, **kernel_kwargs):
    """MCMC.run for one chain: returns (samples [S, D], extras dict, last_state)."""
    init_kernel, sample_kernel = hmc(potential_and_grad, algo=algo)
    z0 = init_to_uniform(seed, chain, dim) if init_params is None else np.asarray(init_params, np.float64)
    state = init_kernel(z0, num_warmup, rng_key=(seed, chain), **kernel_kwargs)
    samples, num_steps, diverging, accept = [], [], [], []
    for _ in range(num_warmup + num_samples):
        state = sample_kernel(state)
        if state.i > num_warmup:
            samples.append(state.z.copy())
            num_steps.append(state.num_steps)
            diverging.append(state.diverging)
            accept.append(state.accept_prob)
    extras = {"num_steps": np.array(num_steps), "diverging": np.array(diverging),
              "accept_prob": np.array(accept)}
    return np.array(samples), extras, state
