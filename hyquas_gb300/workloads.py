"""Seeded synthetic circuits for the benchmark configurations.

The reference's own 28-qubit suite (tests/input/*.qasm) is absent from its
checkout (Git-LFS pointers), so these generators stand in for it with the
shapes the benchmark configurations name.  All randomness comes from one
splitmix64 stream per seed, so every circuit is reproducible on any machine.

A gate is described as a tuple (type, target, control, control2, params) with
reference GateType ordinals; `to_gates` turns a list of them into Gate objects
of the native library, and the oracle consumes the same tuples.
"""
from __future__ import annotations

import math

import numpy as np

# reference GateType ordinals (src/gate.h:7-9)
CCX, CNOT, CY, CZ, CRX, CRY, CU1, CRZ, U1, U2, U3, H, X, Y, Z, S, SDG, T, TDG, RX, RY, RZ = range(22)
SWAP = 28
TWO_PI = 2.0 * math.pi


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014); uniform() has 53 random bits."""

    MASK = (1 << 64) - 1

    def __init__(self, seed: int):
        self.s = seed & self.MASK

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / (1 << 53))

    def below(self, n: int) -> int:
        return self.next() % n

    def shuffle(self, xs: list) -> list:
        xs = list(xs)
        for i in range(len(xs) - 1, 0, -1):
            j = self.below(i + 1)
            xs[i], xs[j] = xs[j], xs[i]
        return xs


def g1(t, q, *params):
    return (t, q, -1, -1, tuple(params))


def g2(t, c, q, *params):
    return (t, q, c, -1, tuple(params))


def plain_u3_cnot(seed: int = 1, n: int = 20, layers: int = 10):
    """The 20-qubit plain-path circuit: per layer U3(theta, phi, lambda) on every qubit with angles
    uniform in [0, 2pi), then CNOT on a random perfect matching."""
    rng = SplitMix64(seed)
    gates = []
    for _ in range(layers):
        for q in range(n):
            gates.append(g1(U3, q, rng.uniform() * TWO_PI, rng.uniform() * TWO_PI,
                            rng.uniform() * TWO_PI))
        perm = rng.shuffle(range(n))
        for i in range(0, n - 1, 2):
            gates.append(g2(CNOT, perm[i], perm[i + 1]))
    return gates


def blocked_u3_cnot(seed: int = 11, n: int = 28, block: int = 7, depth: int = 20, rounds: int = 2):
    """A modular circuit: the qubits form blocks of `block` neighbours; per round every block
    runs `depth` layers of U3 on each of its qubits and CNOTs on alternating neighbour pairs
    inside the block, then one CNOT joins each block to the next.  Deep dense blocks are the
    case the reference's mix mode fuses into one unitary per block (src/compiler.cpp:248-280)."""
    rng = SplitMix64(seed)
    gates = []
    nb = n // block
    for _ in range(rounds):
        for b in range(nb):
            q0 = b * block
            for d in range(depth):
                for q in range(q0, q0 + block):
                    gates.append(g1(U3, q, rng.uniform() * TWO_PI, rng.uniform() * TWO_PI,
                                    rng.uniform() * TWO_PI))
                for q in range(q0 + (d & 1), q0 + block - 1, 2):
                    gates.append(g2(CNOT, q, q + 1))
        for b in range(nb - 1):
            gates.append(g2(CNOT, b * block + block - 1, (b + 1) * block))
    return gates


def grid_couplers(rows: int, cols: int):
    """The 4 alternating coupler patterns of a rows x cols grid: horizontal
    couplers with even / odd column, vertical couplers with even / odd row."""
    q = lambda r, c: r * cols + c
    h_even = [(q(r, c), q(r, c + 1)) for r in range(rows) for c in range(0, cols - 1, 2)]
    h_odd = [(q(r, c), q(r, c + 1)) for r in range(rows) for c in range(1, cols - 1, 2)]
    v_even = [(q(r, c), q(r + 1, c)) for r in range(0, rows - 1, 2) for c in range(cols)]
    v_odd = [(q(r, c), q(r + 1, c)) for r in range(1, rows - 1, 2) for c in range(cols)]
    return [h_even, v_even, h_odd, v_odd]


def grid_random(seed: int = 2, rows: int = 5, cols: int = 6, cycles: int = 20):
    """The random grid circuit: per cycle a random sqrt(X) / sqrt(Y) / T on every qubit (never
    the gate that qubit had in the previous cycle), then CZ on the cycle's
    coupler pattern (4 patterns, alternating).  sqrt(X) = RX(pi/2) and sqrt(Y) =
    RY(pi/2) with the reference's RX/RY matrices."""
    rng = SplitMix64(seed)
    n = rows * cols
    pats = grid_couplers(rows, cols)
    prev = [-1] * n
    gates = []
    for cyc in range(cycles):
        for q in range(n):
            choices = [k for k in range(3) if k != prev[q]]
            k = choices[rng.below(len(choices))]
            prev[q] = k
            if k == 0:
                gates.append(g1(RX, q, math.pi / 2))
            elif k == 1:
                gates.append(g1(RY, q, math.pi / 2))
            else:
                gates.append(g1(T, q))
        for a, b in pats[cyc % 4]:
            gates.append(g2(CZ, a, b))
    return gates


def qft(n: int = 28, swaps: bool = True):
    """The quantum Fourier transform: H and CU1(pi / 2^k) for all n(n-1)/2 pairs, then the final
    qubit-order swaps (as SWAP gates, folded into the layout)."""
    gates = []
    for j in range(n - 1, -1, -1):
        gates.append(g1(H, j))
        for k in range(j - 1, -1, -1):
            gates.append(g2(CU1, k, j, math.pi / (1 << (j - k))))
    if swaps:
        for i in range(n // 2):
            gates.append((SWAP, i, n - 1 - i, -1, ()))
    return gates


def random_state(seed: int, n: int) -> np.ndarray:
    """iid complex Gaussian amplitudes, normalised (numpy PCG64 seeded)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal(1 << n, dtype=np.float32) + 1j * rng.standard_normal(1 << n, dtype=np.float32)
    a = a.astype(np.complex64)
    a /= np.float32(np.sqrt(np.sum(np.abs(a.astype(np.complex128)) ** 2)))
    return a


def ry_rz_cz(rng: SplitMix64, n: int, depth: int):
    """The batched and served circuit body: per layer RY and RZ (angles in [0, 2pi)) on every
    qubit, then CZ on a random perfect matching."""
    gates = []
    for _ in range(depth):
        for q in range(n):
            gates.append(g1(RY, q, rng.uniform() * TWO_PI))
            gates.append(g1(RZ, q, rng.uniform() * TWO_PI))
        perm = rng.shuffle(range(n))
        for i in range(0, n - 1, 2):
            gates.append(g2(CZ, perm[i], perm[i + 1]))
    return gates


def batched(seed: int = 4, count: int = 512, nmin: int = 10, nmax: int = 22, dmin: int = 8,
            dmax: int = 40):
    """A batch of `count` circuits, n uniform in [nmin, nmax], depth uniform in [dmin, dmax]."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        n = nmin + rng.below(nmax - nmin + 1)
        d = dmin + rng.below(dmax - dmin + 1)
        out.append((n, ry_rz_cz(rng, n, d)))
    return out


def served_stream(seed: int = 5, count: int = 200, rate: float = 1000.0, nmin: int = 12,
                  nmax: int = 32, dmin: int = 10, dmax: int = 60):
    """A served stream: Poisson arrivals at `rate` per second; n log-uniform in
    [nmin, nmax]; circuits as in the batch.  Returns (arrival_s, n, gates)."""
    rng = SplitMix64(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += -math.log(1.0 - rng.uniform()) / rate
        n = int(math.floor(math.exp(math.log(nmin) + rng.uniform() * (math.log(nmax + 1) - math.log(nmin)))))
        n = max(nmin, min(nmax, n))
        d = dmin + rng.below(dmax - dmin + 1)
        out.append((t, n, ry_rz_cz(rng, n, d)))
    return out


def to_gates(desc):
    """Gate tuples -> native Gate objects."""
    from . import Gate
    out = []
    for (t, q, c, c2, p) in desc:
        out.append(Gate._make(t, q, c, c2, p))
    return out
