"""Golden fixtures from the reference ops themselves.

Runs on a CUDA machine.  `prepare_reference.sh` must have copied the
reference ops (with the `namespace cuda` -> `namespace refcuda` rename) into
baseline/_ref/ops first.  This script compiles the five reference extensions
directly with nvcc/g++ (each under its own module name, so the three LBP
variants that the reference builds as one `pytorch_cuda_lbp_op` can be loaded
side by side), runs them on seeded inputs from cases.py, and writes one .npz
per case holding the inputs and the reference outputs.

Usage:  python tests/golden/make_golden.py OUT_DIR
The fixtures committed under tests/golden/ were produced by this script.

Every case stays inside the reference kernels' valid range, checked by
reading their index arithmetic: batch 1 (the backward allocates its pairwise
gradient with batch 1), H <= W (the horizontal backward sizes its scratch by W
but indexes it by y), step == 1 for SAD (step != 1 reads one element past the
row), flow windows of at most 109 labels (shared-memory limit).
"""
from __future__ import annotations

import hashlib
import importlib.machinery
import importlib.util
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import cases  # noqa: E402

REF = os.path.join(ROOT, "baseline", "_ref", "ops")
BUILD = os.path.join(ROOT, "baseline", "_ref", "build")

EXTS = {
    "ref_lbp_stereo": ["lbp_stereo/src/lbp.cpp", "lbp_stereo/src/lbp_min_sum_kernel.cu"],
    "ref_lbp_sem_global": ["lbp_semantic_pw/src/lbp.cpp", "lbp_semantic_pw/src/lbp_min_sum_kernel.cu"],
    "ref_lbp_sem_pixel": ["lbp_semantic_pw_pixel/src/lbp.cpp", "lbp_semantic_pw_pixel/src/lbp_min_sum_kernel.cu"],
    "ref_stereo_sad": ["sad/src/stereo_sad.cpp", "sad/src/stereo_sad_kernel.cu"],
    "ref_flow_mp_sad": ["flow_mp_sad/src/flow_mp_sad.cpp", "flow_mp_sad/src/flow_mp_sad_kernel.cu"],
}


def _torch_paths():
    import torch.utils.cpp_extension as ce
    try:
        inc = ce.include_paths(device_type="cuda")
    except TypeError:
        inc = ce.include_paths(cuda=True)
    try:
        lib = ce.library_paths(device_type="cuda")
    except TypeError:
        lib = ce.library_paths(cuda=True)
    return inc, lib


def _stamp(name, srcs):
    h = hashlib.sha256()
    for s in srcs:
        with open(os.path.join(REF, s), "rb") as fh:
            h.update(fh.read())
    import torch
    h.update(torch.__version__.encode())
    return h.hexdigest()


def build_reference(arch="103", names=None):
    """Compiles the reference extensions `names` (default: all five) into
    baseline/_ref/build/<name>.so; an extension whose sources and torch
    version are unchanged since its last build is kept."""
    import torch
    inc, lib = _torch_paths()
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    py_inc = sysconfig.get_paths()["include"]
    abi = int(getattr(torch._C, "_GLIBCXX_USE_CXX11_ABI", 1))
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    links = {}
    for name, srcs in EXTS.items():
        if names is not None and name not in names:
            continue
        stamp = _stamp(name, srcs)
        so = os.path.join(BUILD, name + ".so")
        sp = os.path.join(BUILD, name + ".stamp")
        if os.path.exists(so) and os.path.exists(sp) and open(sp).read() == stamp:
            continue
        incs = ["-I" + os.path.join(REF, "include"), "-I" + py_inc] + ["-I" + p for p in inc]
        defs = [f"-DTORCH_EXTENSION_NAME={name}", "-DTORCH_API_INCLUDE_EXTENSION_H",
                f"-D_GLIBCXX_USE_CXX11_ABI={abi}"]
        objs = []
        for s in srcs:
            src = os.path.join(REF, s)
            obj = os.path.join(BUILD, name + "_" + os.path.basename(s) + ".o")
            objs.append(obj)
            if s.endswith(".cu"):
                cmd = [os.path.join(cuda_home, "bin", "nvcc"), "-c", src, "-o", obj, "-std=c++17",
                       f"-gencode=arch=compute_{arch},code=sm_{arch}",
                       "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
                       "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__",
                       "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-w"] + incs + defs
            else:
                cmd = ["g++", "-c", src, "-o", obj, "-std=c++17", "-O2", "-fPIC", "-w",
                       "-I" + os.path.join(cuda_home, "include")] + incs + defs
            jobs.append(cmd)
        link = ["g++", "-shared", "-o", os.path.join(BUILD, name + ".so")] + objs + \
               ["-L" + p for p in lib] + ["-L" + os.path.join(cuda_home, "lib64")] + \
               ["-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu", "-ltorch_cuda", "-ltorch_python", "-lcudart"] + \
               ["-Wl,-rpath," + p for p in lib] + ["-Wl,-rpath," + os.path.join(cuda_home, "lib64")]
        links[name] = (link, stamp)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])

    with ThreadPoolExecutor(max_workers=min(10, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    for name, (link, stamp) in links.items():
        run(link)
        with open(os.path.join(BUILD, name + ".stamp"), "w") as fh:
            fh.write(stamp)


def load(name):
    path = os.path.join(BUILD, name + ".so")
    loader = importlib.machinery.ExtensionFileLoader(name, path)
    spec = importlib.util.spec_from_file_location(name, path, loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


def T(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda().contiguous()


def N(t):
    return t.detach().cpu().numpy()


def lbp_forward_case(mod, cost, jump, edge, msgs, delta, iters):
    c, j, e = T(cost), T(jump), T(edge)
    m = T(msgs)
    out = {}
    for it in range(iters):
        m, am, sc = mod.forward_minsum(c, j, e, m, int(delta))
        out[f"messages_{it}"] = N(m).copy()
        out[f"argmin_{it}"] = N(am)
        out[f"scale_{it}"] = N(sc)
    return out


def main(outdir):
    import torch
    os.makedirs(outdir, exist_ok=True)
    build_reference()
    st, sg, sp = load("ref_lbp_stereo"), load("ref_lbp_sem_global"), load("ref_lbp_sem_pixel")
    sad, flow = load("ref_stereo_sad"), load("ref_flow_mp_sad")
    written = []

    def save(name, **arrs):
        p = os.path.join(outdir, name + ".npz")
        np.savez_compressed(p, **arrs)
        written.append(p)

    # --- stereo LBP forward -------------------------------------------------
    specs = [
        # name, seed, H, W, L, taps, delta, iters, quantise, msg_init
        ("lbp_stereo_fwd_l32", 11, 12, 16, 32, "scalar", 3, 2, None, "zeros"),
        ("lbp_stereo_fwd_l32_ties", 12, 12, 16, 32, "scalar", 3, 2, 8, "zeros"),
        ("lbp_stereo_fwd_l70_off", 13, 9, 13, 70, "taps8_off", 3, 1, None, "random"),
        ("lbp_stereo_fwd_l33_ties", 14, 7, 9, 33, "taps8", 2, 2, 4, "random_q"),
        ("lbp_stereo_fwd_l20_full", 15, 8, 10, 20, "scalar", 20, 2, 4, "zeros"),
        ("lbp_stereo_fwd_l5_row", 16, 1, 7, 5, "scalar", 3, 1, None, "zeros"),
        ("lbp_stereo_fwd_l1", 17, 4, 5, 1, "scalar", 3, 1, None, "zeros"),
        ("lbp_stereo_fwd_l192", 18, 5, 8, 192, "scalar", 3, 1, None, "zeros"),
    ]
    for name, seed, H, W, L, taps, delta, iters, q, minit in specs:
        g = cases.rng(seed)
        cost = cases.random_cost(g, 1, H, W, L, quantise=q)
        if taps == "scalar":
            jump = cases.stereo_taps(1, H, W, 0.1, 0.5)
        else:
            jump = cases.random_taps8(g, 1, H, W, offset_scale=1.5 if taps == "taps8_off" else 0.0)
            if q:
                jump = (np.round(jump * q) / q).astype(np.float32)
        edge = cases.edge_weights(g, 1, H, W, quantise=q)
        if minit == "zeros":
            msgs = np.zeros((1, 4, H, W, L), np.float32)
        else:
            msgs = cases.random_messages(g, 1, H, W, L, quantise=q if minit == "random_q" else None)
        out = lbp_forward_case(st, cost, jump, edge, msgs, delta, iters)
        save(name, cost=cost, jump=jump, edge=edge, messages_in=msgs, delta=np.int32(delta),
             iters=np.int32(iters), **out)

    # --- stereo LBP forward at the small-config size (96x128x32) -------------
    g = cases.rng(0)
    cost, f0, f1, disp = cases.stereo_cost_from_scene(g, 1, 96, 128, 32, 32)
    jump = cases.stereo_taps(1, 96, 128, 0.1, 0.5)
    edge = np.ones((1, 4, 96, 128), np.float32)
    msgs = np.zeros((1, 4, 96, 128, 32), np.float32)
    out = lbp_forward_case(st, cost, jump, edge, msgs, 3, 1)
    m = out["messages_0"]
    idx = cases.rng(99).choice(m.size, size=20000, replace=False)
    save("lbp_stereo_fwd_c0", cost=cost, delta=np.int32(3), argmin_u8=out["argmin_0"].astype(np.uint8),
         scale=out["scale_0"], msg_idx=idx.astype(np.int64), msg_sample=m.reshape(-1)[idx],
         msg_sha256=np.frombuffer(hashlib.sha256(m.tobytes()).digest(), np.uint8))

    # --- stereo LBP backward (reference adjoint) ------------------------------
    for name, seed, H, W, L, taps in (("lbp_stereo_bwd_l32", 21, 10, 14, 32, "scalar"),
                                      ("lbp_stereo_bwd_l70_off", 22, 9, 13, 70, "taps8_off")):
        g = cases.rng(seed)
        cost = cases.random_cost(g, 1, H, W, L)
        jump = cases.stereo_taps(1, H, W, 0.1, 0.5) if taps == "scalar" else \
            cases.random_taps8(g, 1, H, W, offset_scale=1.5)
        edge = cases.edge_weights(g, 1, H, W)
        msgs = np.zeros((1, 4, H, W, L), np.float32)
        out = lbp_forward_case(st, cost, jump, edge, msgs, 3, 1)
        gin = g.normal(0.0, 1.0, size=(1, 4, H, W, L)).astype(np.float32)
        gc, gj, ge, gm = st.backward_minsum(T(cost), T(jump), T(edge), T(gin), T(out["messages_0"]),
                                            T(out["argmin_0"]), T(out["scale_0"]))
        save(name, cost=cost, jump=jump, edge=edge, delta=np.int32(3), messages=out["messages_0"],
             argmin=out["argmin_0"], scale=out["scale_0"], in_grad=gin, grad_cost=N(gc),
             grad_jump=N(gj), grad_edge=N(ge), grad_messages=N(gm))

    # --- semantic global pairwise -------------------------------------------
    for name, seed, H, W, L, delta in (("lbp_sem_global_l19", 31, 10, 12, 19, 19),
                                       ("lbp_sem_global_l19_trunc", 32, 8, 11, 19, 3)):
        g = cases.rng(seed)
        cost = cases.random_cost(g, 1, H, W, L)
        jump, _ = cases.semantic_global_jump(g, L)
        edge = cases.edge_weights(g, 1, H, W)
        msgs = np.zeros((1, 4, H, W, L), np.float32)
        out = lbp_forward_case(sg, cost, jump, edge, msgs, delta, 2)
        gin = g.normal(0.0, 1.0, size=(1, 4, H, W, L)).astype(np.float32)
        gc, gj, ge, gm = sg.backward_minsum(T(cost), T(jump), T(edge), T(gin), T(out["messages_1"]),
                                            T(out["argmin_1"]), T(out["scale_1"]))
        save(name, cost=cost, jump=jump, edge=edge, messages_in=msgs, delta=np.int32(delta),
             iters=np.int32(2), in_grad=gin, grad_cost=N(gc), grad_jump=N(gj), grad_edge=N(ge),
             grad_messages=N(gm), **out)

    # --- semantic pixel pairwise --------------------------------------------
    g = cases.rng(41)
    H, W, L = 8, 10, 7
    cost = cases.random_cost(g, 1, H, W, L)
    jump, _ = cases.semantic_pixel_jump(g, H, W, L)
    edge = cases.edge_weights(g, 1, H, W)
    msgs = np.zeros((1, 4, H, W, L), np.float32)
    out = lbp_forward_case(sp, cost, jump, edge, msgs, L, 2)
    gin = g.normal(0.0, 1.0, size=(1, 4, H, W, L)).astype(np.float32)
    gc, gj, ge, gm = sp.backward_minsum(T(cost), T(edge), T(gin), T(out["messages_1"]),
                                        T(out["argmin_1"]), T(out["scale_1"]))
    save("lbp_sem_pixel_l7", cost=cost, jump=jump, edge=edge, messages_in=msgs, delta=np.int32(L),
         iters=np.int32(2), in_grad=gin, grad_cost=N(gc), grad_jump=N(gj), grad_edge=N(ge),
         grad_messages=N(gm), **out)

    # --- stereo SAD ------------------------------------------------------------
    for name, seed, C, H, W, lo, hi, q in (("sad_c8_d12", 51, 8, 10, 24, 0, 11, None),
                                          ("sad_c8_neg", 52, 8, 9, 20, -3, 5, None),
                                          ("sad_c8_d4_q", 53, 8, 6, 16, 0, 3, 2)):
        g = cases.rng(seed)
        f0 = g.normal(0, 1, size=(1, C, H, W)).astype(np.float32)
        f1 = g.normal(0, 1, size=(1, C, H, W)).astype(np.float32)
        if q:
            f0 = (np.round(f0 * q) / q).astype(np.float32)
            f1 = (np.round(f1 * q) / q).astype(np.float32)
        vol = sad.forward(T(f0), T(f1), lo, hi, 1.0)
        gin = g.normal(0, 1, size=tuple(vol.shape)).astype(np.float32)
        df0, df1 = sad.backward(T(f0), T(f1), lo, hi, T(gin))
        save(name, f0=f0, f1=f1, min_disp=np.int32(lo), max_disp=np.int32(hi), volume=N(vol),
             in_grad=gin, df0=N(df0), df1=N(df1))

    # --- flow MP-SAD -----------------------------------------------------------
    for name, seed, C, H, W, sws, ou, ov, bu, bv in (("flow_sws6", 61, 4, 10, 12, 6, 0, 0, 0, 0),
                                                    ("flow_sws8_off", 62, 4, 9, 11, 8, -4, 4, 1, 0),
                                                    ("flow_sws5_odd", 63, 3, 7, 9, 5, 0, 0, 0, 0)):
        g = cases.rng(seed)
        f0 = g.normal(0, 1, size=(1, C, H, W)).astype(np.float32)
        f1 = g.normal(0, 1, size=(1, C, H, W)).astype(np.float32)
        cu, cv, us, vs = flow.forward(T(f0), T(f1), sws, ou, ov, bu, bv)
        gu = g.normal(0, 1, size=tuple(cu.shape)).astype(np.float32)
        gv = g.normal(0, 1, size=tuple(cv.shape)).astype(np.float32)
        df0, df1 = flow.backward(T(f0), T(f1), sws, T(gu), T(gv), us, vs)
        save(name, f0=f0, f1=f1, sws=np.int32(sws), offset_u=np.int32(ou), offset_v=np.int32(ov),
             block_u=np.int32(bu), block_v=np.int32(bv), cv_u=N(cu), cv_v=N(cv), u_star=N(us),
             v_star=N(vs), in_grad_u=gu, in_grad_v=gv, df0=N(df0), df1=N(df1))

    torch.cuda.synchronize()
    for p in written:
        print(p, os.path.getsize(p))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py OUT_DIR")
    main(sys.argv[1])
