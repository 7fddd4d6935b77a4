"""Generate the oracle regression fixtures in this directory.

    python tests/golden/make_golden.py

The reference (Fortran + MPI) cannot be compiled here, so these vectors are
outputs of the C oracle (oracle/tam_oracle.c), frozen so that (1) a change to
the oracle shows up as a fixture mismatch and (2) the GPU tests can check the
CUDA library against committed numbers without running the oracle.  Every
case is small enough for the oracle to finish in about a second.

Cases (all FP64, Philox streams keyed by (seed, packet id, stream)):
  coupled_ref_16.npz   reference mode, 16^3, 3000 packets/pass, tophat 8 W,
                       8 outer iterations of src/mcpolar.f90:148-186, seed 2024
  config_layers.npz    config-mode transport, 20x20x16 three-layer slab with an
                       ablated pocket, Gaussian beam, Fresnel, roulette,
                       3000 packets, seed 5 stream 1
  fused_24.npz         config-mode fused heat step, 24x20x16, 30 steps with a
                       closed-form source, Robin top face, Arrhenius
  philox.npz           Philox4x32-10 words for a grid of counters and keys
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# Case definitions shared with the tests.
COUPLED = dict(nx=16, ny=16, nz=16, nphotons=3000, power=8.0, pulse_type=1, seed=2024, iters=8)
LAYERS = dict(nx=20, ny=20, nz=16, half=0.25, radius=0.08, n=3000, seed=5, stream=1,
              mats=[(0.0, 0.0, 0.0, 1.0), (1.0, 200.0, 0.8, 1.4), (0.3, 120.0, 0.9, 1.4), (0.1, 80.0, 0.9, 1.4)])
FUSED = dict(nx=24, ny=20, nz=16, half=0.12, dt=2e-3, steps=30, jscale=2e9)


def layers_grid():
    c = LAYERS
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    g = np.full((nx, ny, nz), 3, dtype=np.uint8, order="F")
    g[:, :, nz - 2:] = 1
    g[:, :, 6:nz - 2] = 2
    g[8:12, 8:12, nz - 3:] = 0
    return g


def fused_source():
    c = FUSED
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    s = np.sin(0.37 * i + 0.11 * j * j + 0.53 * k) * np.cos(0.29 * i * j + 0.07 * k)
    return np.asfortranarray(s * s * c["jscale"])


def philox_inputs():
    ctr = [[i, 3 * i + 1, 0xFFFFFFFF - i, 0x9E3779B9 ^ i] for i in range(16)]
    key = [[0x12345678 + 7 * i, 0xCAFEF00D - i] for i in range(16)]
    return np.array(ctr, dtype=np.uint32), np.array(key, dtype=np.uint32)


def coupled(orc):
    c = COUPLED
    o = orc.RefOracle(orc.ref_params(nx=c["nx"], ny=c["ny"], nz=c["nz"], nphotons=c["nphotons"], power=c["power"],
                                     pulse_type=c["pulse_type"]))
    for _ in range(c["iters"]):
        if o.outer_iteration(c["seed"], nthreads=0) != 0:
            raise RuntimeError("oracle outer iteration failed")
    out = {k: o.arr(k).copy(order="F") for k in ("temp", "jmeanGLOBAL", "tissue", "rhokap", "Q")}
    out["time"] = np.float64(o.st.time)
    out["counter"] = np.int64(o.st.counter)
    o.close()
    return out


def layers(orc):
    c = LAYERS
    d = orc.mc_desc(c["nx"], c["ny"], c["nz"], c["half"], c["half"], c["half"], materials=c["mats"],
                    source_radius=c["radius"])
    jm, tal = orc.mc_transport(d, layers_grid(), c["n"], seed=c["seed"], stream=c["stream"], nthreads=0)
    out = {"jmean": jm}
    for k, v in tal.items():
        out["tally_" + k] = np.float64(v)
    return out


def fused(orc):
    c = FUSED
    nx, ny, nz = c["nx"], c["ny"], c["nz"]
    h = orc.heat_desc(nx, ny, nz, 2 * c["half"] * 1e-2 / nx, 2 * c["half"] * 1e-2 / ny, 2 * c["half"] * 1e-2 / nz,
                      dt=c["dt"])
    shape = (nx, ny, nz)
    T = np.full(shape, 310.15, order="F")
    k = np.full(shape, 0.56, order="F")
    rho = np.full(shape, 1070.0, order="F")
    cp = np.full(shape, 3400.0, order="F")
    Q = np.zeros(shape, order="F")
    om = np.zeros(shape, order="F")
    th = np.zeros(shape + (3,), order="F")
    mat = np.ones(shape, dtype=np.uint8, order="F")
    J = fused_source()
    for s in range(c["steps"]):
        T, _ = orc.fused_step(h, 1.0, (s + 1) * c["dt"], T, k, rho, cp, J, Q, om, th, mat)
    return {"T": T, "omega": om, "thres": th, "mat": mat}


def philox_case(orc):
    ctr, key = philox_inputs()
    words = np.array([orc.philox(list(map(int, ctr[i])), list(map(int, key[i]))) for i in range(len(ctr))],
                     dtype=np.uint32)
    return {"ctr": ctr, "key": key, "words": words}


CASES = {"coupled_ref_16": coupled, "config_layers": layers, "fused_24": fused, "philox": philox_case}


def main():
    import build_oracle

    build_oracle.build()
    import oracle as orc

    orc.load()
    for name, fn in CASES.items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **fn(orc))
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
