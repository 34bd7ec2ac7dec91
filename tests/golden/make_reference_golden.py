"""Golden vectors from the reference's own MATLAB code, run by the MATLAB
interpreter in mlab.py (no MATLAB or Octave exists on this machine).

Every number stored here comes from executing the reference's unmodified
``.m`` files: the models are built by its mesh functions
(fn_rectangular_structured_mesh, fn_set_els_inside_bdry_to_mat,
fn_add_absorbing_layer, fn_add_fluid_solid_interface_els,
fn_isotropic_stiffness_matrix, fn_get_suitable_time_step,
fn_gaussian_pulse) and solved by its entry point fn_BristolFE_v2
(code/fn_BristolFE_v2.m), which assembles K, C, M with
fn_build_global_matrices_v5 and the generated element routines, adds
interface damping, marches with fn_explicit_dynamic_solver_v6 (both
solver_mode strings) or fn_explicit_dynamic_solver_v5 (prescribed
displacements, reaction forces), and reduces field frames with
fn_get_field_output. The CPU path of the reference is used
(use_gpu_if_available = 0, solver_precision 'double').

Cases (small models, a few hundred samples each):
  plate        steel plate 2 x 1 mm at 0.1 mm, absorbers, 'vel at curent
               time step', 'KE' field, two load steps (the second uses the
               first step's wts)
  coupled_lh   water over steel 2 x 2 mm, ASI2D2 interface, absorbers,
               interface damping, dof_to_use [1 2 4], 'vel at last half
               time step', 'mean(u2)' field, monitor pairs that map to no
               DOF (water nodes' displacements)
  coupled_cur  the same model with every DOF, 'vel at curent time step',
               'div(v)' field
  v5           the plate with the v5 solver: forcing plus prescribed
               displacements, reaction forces

Run:  python tests/golden/make_reference_golden.py <reference checkout root>
(or set REFERENCE_ROOT). Writes reference_runs.npz beside this file; the
tests read only that file.
"""
import os
import sys
import time

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import mlab  # noqa: E402

OUT = os.path.join(HERE, "reference_runs.npz")
VEL_CURRENT = "vel at curent time step"
VEL_LAST_HALF = "vel at last half time step"


def interpreter(ref):
    paths = [os.path.join(ref, p) for p in ("code", os.path.join("code", "internal"),
                                            os.path.join("code", "internal", "elements"), "subdoms")]
    stubs = {
        # console progress output and the GPU probe of the reference
        "fn_console_output": lambda ip, a, n: [],
        "fn_test_if_gpu_present_and_working": lambda ip, a, n: [np.array([[0.0]])],
    }
    return mlab.Interp(paths, stubs)


def call(ip, name, *args, nout=1):
    out = mlab.run(ip, name, list(args), nout)
    return out[0] if nout == 1 else out


def to_py(v):
    """MATLAB value -> plain Python/NumPy for storage."""
    if isinstance(v, mlab.Char):
        return str(v)
    if isinstance(v, mlab.Cell):
        return [to_py(x) for x in v.a.reshape(-1, order="F")]
    if isinstance(v, mlab.Struct):
        return {k: to_py(x) for k, x in v.a.reshape(-1)[0].items()}
    if sp.issparse(v):
        return sp.csc_matrix(v)
    return np.asarray(v)


def materials(ip):
    steel = dict(rho=8000.0, D=call(ip, "fn_isotropic_stiffness_matrix", 210e9, 0.3), el_typ="CPE3")
    water = dict(rho=1000.0, D=np.array([[1500.0 ** 2 * 1000.0]]), el_typ="AC2D3")
    return steel, water


def plate_model(ip, steel):
    W, H, h, th = 2e-3, 1e-3, 0.1e-3, 0.3e-3
    mod = call(ip, "fn_rectangular_structured_mesh", np.array([[0, 0], [W, 0], [W, H], [0, H]]), h)
    inner = np.array([[th, th], [W - th, th], [W - th, 2 * H], [th, 2 * H]])
    mod = call(ip, "fn_add_absorbing_layer", mod, inner, th)
    return mod, [steel], h


def coupled_model(ip, steel, water):
    W, H, h, th = 2e-3, 2e-3, 0.1e-3, 0.4e-3
    mod = call(ip, "fn_rectangular_structured_mesh", np.array([[0, 0], [W, 0], [W, H], [0, H]]), h)
    mod = call(ip, "fn_set_els_inside_bdry_to_mat", mod,
               np.array([[-1, H / 2], [W + 1, H / 2], [W + 1, H + 1], [-1, H + 1]]), 2.0)
    inner = np.array([[th, th], [W - th, th], [W - th, 2 * H], [th, 2 * H]])
    mod = call(ip, "fn_add_absorbing_layer", mod, inner, th)
    matls = [steel, water]
    mod = call(ip, "fn_add_fluid_solid_interface_els", mod, mlab.to_m(matls))
    return mod, matls, h


def top_nodes(nds, y):
    return np.nonzero(np.isclose(nds[:, 1], y))[0] + 1.0


def signal(ip, matls, h, n_t, scale=1.0):
    dt = float(np.asarray(call(ip, "fn_get_suitable_time_step", mlab.to_m(matls), h)).reshape(-1)[0]) * scale
    t = np.arange(n_t) * dt
    s = np.asarray(call(ip, "fn_gaussian_pulse", t.reshape(1, -1), 5e6, 5.0))
    return t, s


def cases(ip):
    steel, water = materials(ip)
    out = []
    # plate: two steps, wts, an invalid monitor pair
    mod, matls, h = plate_model(ip, steel)
    nds = to_py(mod)["nds"]
    t, s = signal(ip, matls, h, 300, 0.8)
    top = top_nodes(nds, nds[:, 1].max())
    ctr = top[np.argmin(np.abs(nds[top.astype(int) - 1, 0] - nds[:, 0].max() / 2))]
    mon = top[::2]
    steps = [
        {"load": {"time": t, "frc_nds": np.array([ctr, ctr + 1]), "frc_dfs": np.array([2.0, 2.0]),
                  "frcs": s, "wts": np.array([1.0, 0.5])},
         "mon": {"nds": mon, "dfs": np.full(mon.size, 2.0)}},
        {"load": {"time": t, "frc_nds": np.array([top[3]]), "frc_dfs": np.array([1.0]), "frcs": s},
         "mon": {"nds": mon, "dfs": np.full(mon.size, 1.0)}},
    ]
    opts = dict(dof_to_use=np.array([1.0, 2.0]), use_gpu_if_available=0.0, field_output_every_n_frames=60.0,
                field_output_type="KE", solver_mode=VEL_CURRENT, solver_precision="double",
                damping_power_law=2.0)
    out.append(("plate", mod, matls, steps, opts))
    # coupled model, both modes
    mod, matls, h = coupled_model(ip, steel, water)
    nds = to_py(mod)["nds"]
    t, s = signal(ip, matls, h, 260, 0.8)
    top = top_nodes(nds, nds[:, 1].max())
    ctr = top[np.argmin(np.abs(nds[top.astype(int) - 1, 0] - nds[:, 0].max() / 2))]
    iface = top_nodes(nds, 1e-3)
    # the last pair (a water node's displacement) maps to no DOF: res.dsps
    # keeps a zero row for it only up to the last valid monitor
    mnds = np.concatenate([top[::3], iface[::3], iface[::3], [top[1]]])
    mdfs = np.concatenate([np.full(top[::3].size, 4.0), np.full(iface[::3].size, 4.0),
                           np.full(iface[::3].size, 2.0), [2.0]])
    mnds = np.concatenate([mnds[:2], [top[2]], mnds[2:]])
    mdfs = np.concatenate([mdfs[:2], [1.0], mdfs[2:]])
    steps = [{"load": {"time": t, "frc_nds": np.array([ctr]), "frc_dfs": np.array([4.0]), "frcs": s},
              "mon": {"nds": mnds, "dfs": mdfs}}]
    opts = dict(dof_to_use=np.array([1.0, 2.0, 4.0]), use_gpu_if_available=0.0, field_output_every_n_frames=50.0,
                field_output_type="mean(u2)", solver_mode=VEL_LAST_HALF, solver_precision="double",
                damping_power_law=2.0, interface_damping_factor=0.5)
    out.append(("coupled_lh", mod, matls, steps, opts))
    opts = dict(dof_to_use=np.zeros((0, 0)), use_gpu_if_available=0.0, field_output_every_n_frames=65.0,
                field_output_type="div(v)", solver_mode=VEL_CURRENT, solver_precision="double")
    out.append(("coupled_cur", mod, matls, steps, opts))
    # v5 with prescribed displacements on the plate
    mod, matls, h = plate_model(ip, steel)
    nds = to_py(mod)["nds"]
    t, s = signal(ip, matls, h, 240, 0.5)
    top = top_nodes(nds, nds[:, 1].max())
    dsp = np.zeros((2, t.size))
    dsp[0] = 1e-9 * s.reshape(-1)
    dsp[1] = -0.5e-9 * np.roll(s.reshape(-1), 7)
    steps = [{"load": {"time": t, "frc_nds": np.array([top[4]]), "frc_dfs": np.array([2.0]), "frcs": s,
                       "dsp_nds": np.array([top[10], top[12]]), "dsp_dfs": np.array([2.0, 1.0]), "dsps": dsp},
              "mon": {"nds": np.concatenate([top[::2], [top[10]]]),
                      "dfs": np.concatenate([np.full(top[::2].size, 2.0), [2.0]])}}]
    opts = dict(dof_to_use=np.array([1.0, 2.0]), use_gpu_if_available=0.0, field_output_every_n_frames=75.0,
                field_output_type="KE", solver_mode=VEL_CURRENT, solver_precision="double",
                dynamic_solver_version="v5")
    out.append(("v5", mod, matls, steps, opts))
    return out


def store(rec, key, v):
    if sp.issparse(v):
        v = sp.csc_matrix(v)
        rec[key + ".data"] = v.data
        rec[key + ".indices"] = v.indices.astype(np.int64)
        rec[key + ".indptr"] = v.indptr.astype(np.int64)
        rec[key + ".shape"] = np.array(v.shape, np.int64)
    elif isinstance(v, str):
        rec[key] = np.array(v)
    elif isinstance(v, list):
        rec[key] = np.array([str(x) for x in v])
    elif isinstance(v, dict):
        for k, x in v.items():
            store(rec, key + "." + k, x)
    elif v is None:
        pass
    else:
        rec[key] = np.asarray(v)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT", "")
    if not os.path.isfile(os.path.join(ref, "code", "fn_BristolFE_v2.m")):
        print("reference checkout not found (pass its root as the first argument)")
        sys.exit(1)
    ip = interpreter(ref)
    rec = {}
    for name, mod, matls, steps, opts in cases(ip):
        t0 = time.time()
        res, mats = call(ip, "fn_BristolFE_v2", mod, mlab.to_m(matls),
                         mlab.Cell(np.array([[mlab.to_m(st) for st in steps]], dtype=object)),
                         mlab.to_m(opts), nout=2)
        store(rec, name + ".mod", to_py(mod))
        for k, m in enumerate(matls):
            store(rec, name + ".matl%d" % k, {"rho": m["rho"], "D": np.asarray(m["D"]), "el_typ": m["el_typ"]})
        rec[name + ".n_matls"] = np.array(len(matls))
        for k, st in enumerate(steps):
            store(rec, name + ".step%d" % k, st)
        rec[name + ".n_steps"] = np.array(len(steps))
        store(rec, name + ".opts", opts)
        store(rec, name + ".mats", to_py(mats))
        rl = to_py(res)
        for k, r in enumerate(rl):
            store(rec, name + ".res%d" % k, r)
        print("%-12s %6d DOF  %.1f s" % (name, to_py(mats)["K"].shape[0], time.time() - t0))
    np.savez_compressed(OUT, **rec)
    print("wrote", OUT, "%.0f kB" % (os.path.getsize(OUT) / 1e3))


if __name__ == "__main__":
    main()
