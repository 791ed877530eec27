"""Regenerate the golden fixtures of the CPU oracle (tests/golden/*.npz).

The reference cannot run here (Julia is absent), so these vectors are the
oracle's output on small seeded ensembles of each workload, in both rounding
modes.  They pin the oracle against unintended change; its agreement with the
reference rests on the analytic and relational tests of test_oracle.py and on
the order conditions of test_tableaus.py.

Usage: python tests/golden/make_golden.py  (writes next to this file)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
T_ARENSTORF = 17.0652165601579625588917206249


def lorenz(n, seed, rho_hi=30.0, u0=None):
    rng = np.random.default_rng(seed)
    if u0 is None:
        u = rng.uniform(-1, 1, (3, n))
        u[2] += 20
    else:
        u = np.tile(np.asarray(u0, float)[:, None], (1, n))
    p = np.stack([np.full(n, 10.0), rng.uniform(0, rho_hi, n), np.full(n, 8 / 3)])
    return u, p


def vdp(n, seed):
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10), n))[None, :]
    return rng.uniform(-2, 2, (2, n)), mu


def r3bp(n, seed):
    rng = np.random.default_rng(seed)
    return (np.array([0.994, 0.0, 0.0, -2.00158510637908])[:, None] + rng.normal(0, 1e-4, (4, n)),
            np.full((1, n), 0.012277471))


def kuramoto(n, seed, D=12):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 2 * np.pi, (D, n)), np.vstack([rng.normal(0, 1, (D, n)), rng.uniform(0, 4, (1, n))])


CASES = {
    "tsit5_lorenz_fixed_dev": dict(alg="Tsit5", rhs="lorenz", inputs=("lorenz", 32, 1, 21.0, (1, 0, 0)),
                                   tspan=(0, 1), dt=0.01, rounding="device"),
    "tsit5_lorenz_fixed_ref": dict(alg="Tsit5", rhs="lorenz", inputs=("lorenz", 32, 1, 21.0, (1, 0, 0)),
                                   tspan=(0, 1), dt=0.01, rounding="ref"),
    "atsit5_lorenz_dev": dict(alg="ATsit5", rhs="lorenz", inputs=("lorenz", 32, 2, 30.0, None), tspan=(0, 10),
                              dt=0.1, abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 10, 100), rounding="device"),
    "atsit5_lorenz_dev_ctrl32": dict(alg="ATsit5", rhs="lorenz", inputs=("lorenz", 32, 2, 30.0, None),
                                     tspan=(0, 10), dt=0.1, abstol=1e-8, reltol=1e-6,
                                     saveat=np.linspace(0, 10, 100), rounding="device", controller="fp32"),
    "atsit5_lorenz_ref": dict(alg="ATsit5", rhs="lorenz", inputs=("lorenz", 32, 2, 30.0, None), tspan=(0, 10),
                              dt=0.1, abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 10, 100), rounding="ref"),
    "avern7_vdp_dev": dict(alg="AVern7", rhs="vanderpol", inputs=("vdp", 16, 3), tspan=(0, 20), dt=0.1,
                           abstol=1e-10, reltol=1e-8, saveat=np.linspace(0, 20, 200), rounding="device"),
    "avern9_r3bp_dev": dict(alg="AVern9", rhs="r3bp", inputs=("r3bp", 16, 4), tspan=(0, T_ARENSTORF), dt=0.1,
                            abstol=1e-12, reltol=1e-12, rounding="device"),
    "avern9_r3bp_fp32k": dict(alg="AVern9", rhs="r3bp", inputs=("r3bp", 16, 4), tspan=(0, T_ARENSTORF), dt=0.1,
                              abstol=1e-7, reltol=1e-7, precision="fp32_kahan", rounding="device"),
    "atsit5_kuramoto_ref": dict(alg="ATsit5", rhs="kuramoto", inputs=("kuramoto", 8, 5), tspan=(0, 50), dt=0.1,
                                abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 50, 50), rounding="ref"),
    "atsit5_kuramoto_dev": dict(alg="ATsit5", rhs="kuramoto", inputs=("kuramoto", 8, 5), tspan=(0, 50), dt=0.1,
                                abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 50, 50), rounding="device"),
    "atsit5_kuramoto_r_dev": dict(alg="ATsit5", rhs="kuramoto", inputs=("kuramoto", 8, 5), tspan=(0, 50), dt=0.1,
                                  abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 50, 50), rounding="device",
                                  output="kuramoto_r"),
}


def make_inputs(spec):
    kind = spec[0]
    if kind == "lorenz":
        return lorenz(spec[1], spec[2], spec[3], spec[4])
    if kind == "vdp":
        return vdp(spec[1], spec[2])
    if kind == "r3bp":
        return r3bp(spec[1], spec[2])
    return kuramoto(spec[1], spec[2])


def run_case(po, case, inputs=None):
    """Solve a case with the oracle; `inputs` = (u0, p) overrides the generated inputs."""
    c = dict(case)
    u0, p = make_inputs(c.pop("inputs")) if inputs is None else inputs
    if inputs is not None:
        c.pop("inputs")
    alg, rhs, tspan, dt = c.pop("alg"), c.pop("rhs"), c.pop("tspan"), c.pop("dt")
    return po.solve(alg, rhs, u0, p, tspan, dt, **c)


def main():
    sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
    import pyoracle as po
    for name, case in CASES.items():
        # the inputs are stored with the outputs: numpy's exp/log (used for log-uniform parameters
        # and normal samples) may round differently on other machines, so consumers use these, and a
        # regeneration keeps the committed ones
        path = os.path.join(HERE, name + ".npz")
        if os.path.exists(path):
            old = np.load(path)
            u0, p = old["u0"], old["p"]
        else:
            u0, p = make_inputs(case["inputs"])
        out = run_case(po, case, (u0, p))
        keep = {k: out[k] for k in ("u_final", "naccept", "nreject", "retcode")}
        if out["us"] is not None:
            keep["us"] = out["us"]
        keep["u0"], keep["p"] = u0, p
        np.savez_compressed(path, **keep)
        print(name, {k: v.shape for k, v in keep.items()})


if __name__ == "__main__":
    main()
