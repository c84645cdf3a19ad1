"""Trains the learned star-pressure proposal on the GPU and evaluates it.

    python phd-2d-gfm_gb300/train_pstar.py [--n 4194304] [--epochs 20] [--eval]

Training data (the learned-guess configuration): n two-material Riemann
problems drawn on the device from its distribution (gamma in [1.09, 4.4],
pinf in {0, 6e8}, pressure ratio log-U[1e-3, 1e5], density ratio
log-U[1e-3, 1e3], velocity jump U[-3, 3] sound speeds) with targets from the
exact FP64 solver (gfm_mlp_generate), plus the gated interface problems the
solver itself meets in a run of the underwater explosion and of strong-shock
members of the batched shock-bubble family (gfm_capture_interface_problems).
The network (10 -> 64 -> 64 -> 64 -> 1, SiLU) is trained by the library's
own kernels (gfm_mlp_train: forward, backward and Adam in FP32) and saved to
data/pstar_mlp.f32 (9089 little-endian floats) with a record of the run in
data/pstar_mlp.json.

--eval runs the plain and the learned paths side by side on the
shock-bubble scaled to 2000 x 800 (2000 steps) and the 800 x 800 underwater
explosion (1500 steps) and records, per path, the Newton iterations per
interface solve, the solves that started from the proposal, the time per
step and the relative L1 difference of the end fields (data/pstar_mlp_eval.json).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import gfm_gb300 as g  # noqa: E402

DATA = os.path.join(HERE, "data")
WEIGHTS = os.path.join(DATA, "pstar_mlp.f32")
RECORD = os.path.join(DATA, "pstar_mlp.json")
EVAL = os.path.join(DATA, "pstar_mlp_eval.json")

# strong-shock members of the batched family whose interface problems are captured
CAPTURE_MEMBERS = [(128, 128, 2.61, 1.2, 0.3, 0.2), (192, 128, 2.13, 1.5, 5.0, 0.25), (448, 192, 2.91, 1.1, 0.15, 0.2)]


def load(path=WEIGHTS):
    """An MLP with the saved weights, or None when they are absent."""
    if not os.path.exists(path):
        return None
    p = np.fromfile(path, dtype="<f4")
    if p.size != g.lib().gfm_mlp_param_count():
        raise ValueError("%s holds %d floats, not %d" % (path, p.size, g.lib().gfm_mlp_param_count()))
    m = g.MLP(seed=1)
    m.set_params(p)
    return m


def capture(X, Y, offset, cap, count):
    """Gated interface problems of solver runs appended to X, Y from offset."""
    import torch
    runs = [("case", "underwater_explosion_sg", 200, 200, "realGFM", 200)]
    runs += [("member", p, None, None, "riemannGFM", 150) for p in CAPTURE_MEMBERS]
    for kind, a, nx, ny, gfm, nsteps in runs:
        if kind == "case":
            desc, T = g.case_params("twofluid", a, nx, ny)
            U1, U2, phi = g.case_init("twofluid", a, desc)
            m = g.method(gfm=gfm, CFL=0.5, T=T, reinit_every=5)
        else:
            desc, T, U1, U2, phi = g.shock_bubble_case(*a)
            m = g.method(gfm=gfm, CFL=0.6, T=T)
        ctx = g.Context(desc, two_fluid=True)
        ctx.upload(U1, U2, phi)
        ctx.capture_interface_problems(X[offset:].data_ptr(), Y[offset:].data_ptr(), cap, count.data_ptr())
        ctx.step(m, nsteps)
        ctx.capture_interface_problems(None, None, 0, None)
        torch.cuda.synchronize()
        ctx.close()
    return min(int(count.item()), cap)


def held_out_iterations(mlp, n=1 << 16, seed=0xE7A1):
    """Newton iterations per solve on held-out problems of the training
    distribution (air | stiffened water, strong waves), from the two-shock
    guess and from the proposal, and the largest relative p* difference."""
    import torch
    rng = np.random.default_rng(seed)
    gL, qL, gR, qR = 1.4, 0.0, 4.4, 6e8
    pL = 10 ** rng.uniform(3, 8, n)
    pR = pL * np.exp(rng.uniform(np.log(1e-3), np.log(1e5), n))
    rL = 10 ** rng.uniform(-1, 3, n)
    rR = rL * np.exp(rng.uniform(np.log(1e-3), np.log(1e3), n))
    cL, cR = np.sqrt(gL * (pL + qL) / rL), np.sqrt(gR * (pR + qR) / rR)
    du = rng.uniform(-2.0, 1.0, n) * 0.5 * (cL + cR)

    def cons(g_, q, rho, u, p):
        return np.stack([rho, rho * u, np.zeros_like(rho), (p + g_ * q) / (g_ - 1.0) + 0.5 * rho * u * u], 1)

    UL = torch.from_numpy(np.ascontiguousarray(cons(gL, qL, rL, -0.5 * du, pL))).cuda()
    UR = torch.from_numpy(np.ascontiguousarray(cons(gR, qR, rR, 0.5 * du, pR))).cuda()
    res = {}
    for net in (False, True):
        out = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
        its = torch.zeros(n, dtype=torch.int32, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        mlp.rs_mixed(gL, qL, gR, qR, UL.data_ptr(), UR.data_ptr(), n, out.data_ptr(), its.data_ptr(), st.data_ptr(),
                     use_net=net)
        torch.cuda.synchronize()
        res[net] = (out.cpu().numpy()[:, 0], its.cpu().numpy())
    vac = (2.0 / (gL - 1.0)) * cL + (2.0 / (gR - 1.0)) * cR <= du
    ok = ~vac & np.isfinite(res[False][0]) & np.isfinite(res[True][0])
    rel = np.abs(res[True][0] - res[False][0]) / (np.abs(res[False][0]) + 1e-6 * np.maximum(pL, pR))
    return {"problems": int(ok.sum()), "newton_per_solve_two_shock": float(res[False][1][ok].mean()),
            "newton_per_solve_learned": float(res[True][1][ok].mean()), "max_rel_pstar_diff": float(rel[ok].max())}


def train(n, epochs, batch, lr, seed):
    import torch
    cap = 1 << 20
    X = torch.empty((n + cap, 10), dtype=torch.float32, device="cuda")
    Y = torch.empty(n + cap, dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    got = g.mlp_generate(seed, n, X.data_ptr(), Y.data_ptr())
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    n_cap = capture(X, Y, got, cap, count)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    mlp = g.MLP(seed=seed + 1)
    t0 = time.perf_counter()
    losses = mlp.train(X.data_ptr(), Y.data_ptr(), got + n_cap, epochs=epochs, batch=batch, lr=lr, seed=seed + 2)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    record = {"synthetic_problems": got, "captured_problems": n_cap, "epochs": epochs, "batch": batch, "lr": lr,
              "seed": seed, "data_seconds": round(t_data, 2), "train_seconds": round(t_train, 2),
              "loss_per_epoch": [float(x) for x in losses],
              "network": "10 -> 64 -> 64 -> 64 -> 1 SiLU, FP32 training (gfm_mlp_train), BF16 tensor-core inference"}
    return mlp, record


def evaluate(mlp, name, desc, U1, U2, phi, m, nsteps):
    """Plain and learned runs of nsteps from the same state."""
    import torch
    out, rec = {}, {}
    for learned in (False, True):
        ctx = g.Context(desc, two_fluid=True)
        if learned:
            ctx.set_mlp(mlp)
        ctx.upload(U1, U2, phi)
        solves = iters = proposed = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(nsteps):
            ctx.step(m, 1)
            s = ctx.interface_stats()
            solves += s["solves"]
            iters += s["newton_iters"]
            proposed += s["proposed"]
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        # step time without the per-step statistics read-back
        ctx2 = g.Context(desc, two_fluid=True)
        if learned:
            ctx2.set_mlp(mlp)
        ctx2.upload(U1, U2, phi)
        ctx2.step(m, 3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k = min(nsteps, 200)
        e0.record()
        ctx2.step(m, k)
        e1.record()
        torch.cuda.synchronize()
        ctx2.close()
        out[learned] = ctx.download()
        rec["learned" if learned else "plain"] = {
            "interface_solves": solves, "newton_iters": iters, "newton_per_solve": iters / max(1, solves),
            "from_proposal": proposed, "ms_per_step": e0.elapsed_time(e1) / k, "status": ctx.status(),
            "wall_seconds_with_statistics": round(el, 2)}
        ctx.close()
    gc = desc.numGC
    rel = 0.0
    for a, b in zip(out[True], out[False]):
        ra, rb = a[..., gc:-gc, gc:-gc], b[..., gc:-gc, gc:-gc]
        rel = max(rel, float(np.abs(ra - rb).sum() / max(np.abs(rb).sum(), 1e-300)))
    rec["max_rel_l1_learned_vs_plain"] = rel
    rec["bit_identical"] = all(np.array_equal(a, b) for a, b in zip(out[True], out[False]))
    rec["steps"] = nsteps
    rec["workload"] = name
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 22)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0x6F4D)
    ap.add_argument("--eval", action="store_true")
    ap.add_argument("--eval-only", action="store_true", help="evaluate the saved weights")
    a = ap.parse_args()
    os.makedirs(DATA, exist_ok=True)
    if a.eval_only:
        mlp = load()
    else:
        mlp, record = train(a.n, a.epochs, a.batch, a.lr, a.seed)
        record["held_out"] = held_out_iterations(mlp)
        mlp.params().astype("<f4").tofile(WEIGHTS)
        json.dump(record, open(RECORD, "w"), indent=1)
        print(json.dumps({k: v for k, v in record.items() if k != "loss_per_epoch"}))
    if a.eval or a.eval_only:
        res = []
        desc, T = g.case_params("twofluid", "shock_bubble", 2000, 800)
        U1, U2, phi = g.case_init("twofluid", "shock_bubble", desc)
        res.append(evaluate(mlp, "shock_bubble_2000x800_riemannGFM (C2 scaled)", desc, U1, U2, phi,
                            g.method(gfm="riemannGFM", CFL=0.6, T=T), 2000))
        desc, T = g.case_params("twofluid", "underwater_explosion_sg", 800, 800)
        U1, U2, phi = g.case_init("twofluid", "underwater_explosion_sg", desc)
        res.append(evaluate(mlp, "underwater_explosion_800x800_realGFM", desc, U1, U2, phi,
                            g.method(gfm="realGFM", CFL=0.5, T=T, reinit_every=5), 1500))
        json.dump(res, open(EVAL, "w"), indent=1)
        for r in res:
            print(json.dumps(r))
    mlp.close()


if __name__ == "__main__":
    main()
