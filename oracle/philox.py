"""Philox4x32-10 and the random-stream layout (oracle side, test infrastructure).

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11).  Each call maps a
128-bit counter and a 64-bit key to four 32-bit words; there is no sequential
state, so a chain's draws depend only on *where* they are taken, never on the
order in which the GPU schedules chains.  The CUDA kernels implement the same
function (``numpyro_gb300/csrc/philox.cuh``) and the same address layout, so
the oracle and the device consume bit-identical uniforms.

Stream address layout (one Philox call = 4 words):

    key     = (seed & 0xffffffff, seed >> 32)
    counter = (chain, n, (purpose << 24) | idx, sub)

    purpose MOMENTUM  (0): n = transition index, idx = block k; the 4 words
                           give latent coordinates 4k..4k+3 through two
                           Box-Muller pairs (numpyro hmc.py:92-110 draws the
                           momentum once per transition, hmc.py:475-481).
    purpose DOUBLING  (1): n = transition, idx = tree depth before the doubling;
                           word 0 -> direction (hmc_util.py:1161-1162),
                           word 1 -> biased transition (hmc_util.py:936 -> :804).
    purpose LEAF      (2): n = transition, idx = depth, sub = leaf index j >= 1
                           inside the subtree; word 0 -> uniform transition
                           (hmc_util.py:1020-1032 -> :804).
    purpose INIT      (3): n = attempt, idx = block k; init_to_uniform(radius=2)
                           (numpyro/infer/initialization.py, infer/util.py:456-463).
    purpose HMC_ACCEPT(4): n = transition; word 0 -> Metropolis accept of
                           fixed-length HMC (hmc.py:407).
    purpose HEURISTIC (5): n = transition at which the search runs (or
                           0xffffffff at init), idx = block k, sub = trial;
                           momentum of find_reasonable_step_size trials
                           (hmc_util.py:314-384).

Uniforms are u = (word >> 8) * 2**-24, exactly representable in float32 and
float64, so a Bernoulli(p) draw ``u < p`` (JAX semantics) takes the same value
on CPU and GPU whenever p agrees.
"""
import numpy as np

PHILOX_M0 = np.uint64(0xD2511F53)
PHILOX_M1 = np.uint64(0xCD9E8D57)
PHILOX_W0 = np.uint32(0x9E3779B9)
PHILOX_W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

MOMENTUM, DOUBLING, LEAF, INIT, HMC_ACCEPT, HEURISTIC = 0, 1, 2, 3, 4, 5
INIT_TRANSITION = 0xFFFFFFFF


def philox4x32_10(counter, key):
    """Vectorised Philox4x32-10.

    counter: uint32 array (..., 4); key: uint32 array (..., 2) broadcastable.
    Returns uint32 array (..., 4).
    """
    c = np.asarray(counter, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    c0, c1, c2, c3 = (c[..., i].astype(np.uint64) for i in range(4))
    k0 = np.broadcast_to(k[..., 0], c[..., 0].shape).astype(np.uint64)
    k1 = np.broadcast_to(k[..., 1], c[..., 0].shape).astype(np.uint64)
    for rnd in range(10):
        p0 = PHILOX_M0 * c0
        p1 = PHILOX_M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c0, c1, c2, c3 = (
            hi1 ^ c1 ^ k0,
            lo1,
            hi0 ^ c3 ^ k1,
            lo0,
        )
        if rnd < 9:
            k0 = (k0 + np.uint64(PHILOX_W0)) & MASK32
            k1 = (k1 + np.uint64(PHILOX_W1)) & MASK32
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def seed_key(seed):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32)


def words_to_uniform(w):
    """(word >> 8) * 2**-24 in [0, 1), exact in float32 and float64."""
    return (np.asarray(w, dtype=np.uint32) >> np.uint32(8)).astype(np.float64) * (2.0 ** -24)


def draw(seed, chain, n, purpose, idx, sub=0):
    ctr = np.array(
        [chain & 0xFFFFFFFF, n & 0xFFFFFFFF, ((purpose << 24) | idx) & 0xFFFFFFFF, sub & 0xFFFFFFFF],
        dtype=np.uint32,
    )
    return philox4x32_10(ctr, seed_key(seed))


def uniform(seed, chain, n, purpose, idx, sub=0, word=0):
    return float(words_to_uniform(draw(seed, chain, n, purpose, idx, sub)[word]))


def box_muller(u0, u1):
    """Two standard normals from two uniforms in [0, 1) (Box and Muller, 1958)."""
    rad = np.sqrt(-2.0 * np.log1p(-u0))
    ang = 2.0 * np.pi * u1
    return rad * np.cos(ang), rad * np.sin(ang)


def normals(seed, chain, n, purpose, dim, sub=0):
    """`dim` standard normals at (chain, n, purpose, block k, sub) for k = 0.."""
    nblk = (dim + 3) // 4
    ctr = np.zeros((nblk, 4), dtype=np.uint32)
    ctr[:, 0] = chain & 0xFFFFFFFF
    ctr[:, 1] = n & 0xFFFFFFFF
    ctr[:, 2] = (purpose << 24) | np.arange(nblk, dtype=np.uint32)
    ctr[:, 3] = sub & 0xFFFFFFFF
    u = words_to_uniform(philox4x32_10(ctr, seed_key(seed)))
    a0, a1 = box_muller(u[:, 0], u[:, 1])
    b0, b1 = box_muller(u[:, 2], u[:, 3])
    out = np.stack([a0, a1, b0, b1], axis=-1).reshape(-1)
    return out[:dim]


def uniforms_block(seed, chain, n, purpose, dim, sub=0):
    """`dim` uniforms in [0,1) at consecutive blocks (used by INIT)."""
    nblk = (dim + 3) // 4
    ctr = np.zeros((nblk, 4), dtype=np.uint32)
    ctr[:, 0] = chain & 0xFFFFFFFF
    ctr[:, 1] = n & 0xFFFFFFFF
    ctr[:, 2] = (purpose << 24) | np.arange(nblk, dtype=np.uint32)
    ctr[:, 3] = sub & 0xFFFFFFFF
    return words_to_uniform(philox4x32_10(ctr, seed_key(seed))).reshape(-1)[:dim]
