"""The FP64 SR layer (vmc_gb300.qgt / preconditioners, plain torch) against the oracle, and the
multi-rank reductions with 2 gloo ranks on CPU."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import peps as oracle
from oracle import sr as osr
from tests.helpers import uniform_init_tensors
from vmc_gb300 import qgt as gq
from vmc_gb300.distributed import gather_jacobian, global_energy, parameter_space_qgt, shard_chains
from vmc_gb300.operators import LocalHamiltonian
from vmc_gb300.preconditioners import DirectSolve, QRSolve, SRPreconditioner, reorder_updates


class _Model:
    """The attributes SRPreconditioner reads from a PEPS (shape, bond_dim, phys_dim, unpack)."""

    def __init__(self, shape, D, d, tensors):
        self.shape, self.bond_dim, self.phys_dim = shape, D, d
        self.tensors = [[torch.as_tensor(t, dtype=torch.float32) for t in row] for row in tensors]

    def unpack(self, flat):
        out, off = [], 0
        for row in self.tensors:
            r = []
            for t in row:
                r.append(flat[off:off + t.numel()].reshape(t.shape))
                off += t.numel()
            out.append(r)
        return out


def _data(n=48, seed=0):
    shape, D = (2, 3), 2
    T = uniform_init_tensors(shape, D, seed=seed)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    rng = np.random.default_rng(seed)
    cfg = rng.integers(0, 2, size=(n, 6))
    amps, grads, p = oracle.value_and_grad(model, cfg)
    e = rng.standard_normal(n)
    return shape, D, T, model, grads / amps[:, None], p, e


@pytest.mark.parametrize("space", ["param", "sample"])
def test_torch_sr_matches_oracle(space):
    shape, D, T, om, o, p, e = _data()
    sd = oracle.sliced_dims(om)
    pps = oracle.params_per_site(om)
    x_ref, m_ref = osr.sr_apply(o, p, e, pps=pps, sliced_dims=sd, n_samples=o.shape[0], diag_shift=1e-3,
                            grad_factor=-1.0, space=osr.ParameterSpace() if space == "param" else osr.SampleSpace())
    pre = SRPreconditioner(space=gq.ParameterSpace() if space == "param" else gq.SampleSpace(), diag_shift=1e-3)
    model = _Model(shape, D, 2, T)
    upd, metrics = pre.apply(model, model.tensors, torch.zeros((o.shape[0], 6)), torch.as_tensor(o),
                             torch.as_tensor(p), torch.as_tensor(e), grad_factor=-1.0)
    flat = torch.cat([u.reshape(-1) for row in upd for u in row]).double().numpy()
    assert np.linalg.norm(flat - x_ref) / np.linalg.norm(x_ref) < 1e-5  # float32 output
    assert abs(float(metrics["residual_error"]) - m_ref["residual_error"]) < 1e-8 * max(1.0, m_ref["residual_error"])


class _ComplexModel(_Model):
    def __init__(self, shape, D, d, tensors):
        self.shape, self.bond_dim, self.phys_dim = shape, D, d
        self.dtype = torch.complex64
        self.tensors = [[torch.as_tensor(t, dtype=torch.complex64) for t in row] for row in tensors]


@pytest.mark.parametrize("space", ["param", "sample"])
@pytest.mark.parametrize("grad_factor", [-1.0, -1.0j])
def test_complex_sr_matches_oracle(space, grad_factor):
    """Complex parameters: complex O, complex E_loc, imaginary (-1) and real (-i) time; no 2 Re(x)."""
    from tests.helpers import complex_tensors

    shape, D = (2, 3), 2
    T = complex_tensors(shape, D, seed=4)
    model = oracle.PEPS(T, shape, D, strategy=oracle.NoTruncation())
    rng = np.random.default_rng(7)
    cfg = rng.integers(0, 2, size=(40, 6))
    amps, grads, p = oracle.value_and_grad(model, cfg)
    o = grads / amps[:, None]
    e = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    sd = oracle.sliced_dims(model)
    x_ref, _ = osr.sr_apply(o, p, e, pps=oracle.params_per_site(model), sliced_dims=sd, n_samples=40,
                            diag_shift=1e-3, grad_factor=grad_factor, real_params=False,
                            space=osr.ParameterSpace() if space == "param" else osr.SampleSpace())
    pre = SRPreconditioner(space=gq.ParameterSpace() if space == "param" else gq.SampleSpace(), diag_shift=1e-3)
    m = _ComplexModel(shape, D, 2, T)
    upd, _ = pre.apply(m, m.tensors, torch.zeros((40, 6)), torch.as_tensor(o), torch.as_tensor(p),
                       torch.as_tensor(e), grad_factor=grad_factor)
    flat = torch.cat([u.reshape(-1) for row in upd for u in row]).to(torch.complex128).numpy()
    assert upd[0][0].dtype == torch.complex64
    assert np.linalg.norm(flat - x_ref) / np.linalg.norm(x_ref) < 1e-5


def test_sample_space_gram_blocked_equals_dense():
    shape, D, T, om, o, p, e = _data(64, 3)
    sd = oracle.sliced_dims(om)
    jac = gq.SlicedJacobian(torch.as_tensor(o), torch.as_tensor(p), sd, gq.SliceOrdering())
    t16 = gq.QGT(jac, gq.SampleSpace(), n_blocks=16).to_dense()
    ref = osr.to_dense(osr.SlicedJacobian(o, p, sd, osr.SliceOrdering()), osr.SampleSpace())
    assert np.allclose(t16.numpy(), ref, rtol=1e-10, atol=1e-12)
    s = gq.QGT(jac, gq.ParameterSpace()).to_dense()
    ref_s = osr.to_dense(osr.SlicedJacobian(o, p, sd, osr.SliceOrdering()), osr.ParameterSpace())
    assert np.allclose(s.numpy(), ref_s, rtol=1e-10, atol=1e-12)
    v = np.random.default_rng(0).standard_normal(s.shape[0])
    assert np.allclose((gq.QGT(jac, gq.ParameterSpace()) @ torch.as_tensor(v)).numpy(), ref_s @ v,
                       rtol=1e-9, atol=1e-12)


def test_reorder_and_qr_solve(emu_lib):
    shape, D, T, om, o, p, e = _data(40, 5)
    sd = oracle.sliced_dims(om)
    pps = tuple(oracle.params_per_site(om))
    x = np.arange(2 * sum(pps), dtype=np.float64)
    assert np.array_equal(reorder_updates(gq.SliceOrdering(), torch.as_tensor(x), pps, sd).numpy(),
                          osr.reorder_updates(osr.SliceOrdering(), x, pps, sd))
    _, grads_full, _ = oracle.value_and_grad(om, np.random.default_rng(5).integers(0, 2, (40, 6)),
                                             full_gradient=True)
    dv = np.random.default_rng(6).standard_normal(40)
    from vmc_gb300.preconditioners import _qr_solve

    xq, mq = _qr_solve(gq.Jacobian(torch.as_tensor(grads_full)), torch.as_tensor(dv), None, True, lib=emu_lib)
    xr, mr = osr.qr_solve(osr.Jacobian(grads_full), dv)
    assert mq["rank"] == mr["rank"]
    assert np.allclose(xq.numpy(), xr, rtol=1e-8, atol=1e-10)


def test_solvers_match():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((20, 20))
    a = a.T @ a + 0.3 * np.eye(20)
    b = rng.standard_normal(20)
    ref = np.linalg.solve(a, b)
    A, B = torch.as_tensor(a), torch.as_tensor(b)
    for f in (gq.solve_cholesky, gq.solve_svd, lambda m, r: gq.solve_cg(m, r, tol=1e-12)):
        assert np.linalg.norm(f(A, B).numpy() - ref) / np.linalg.norm(ref) < 1e-8


def test_shard_chains_cover_everything():
    for n, ws in [(4096, 8), (100, 3), (5, 8)]:
        spans = [shard_chains(n, ws, r) for r in range(ws)]
        assert sum(c for _, c in spans) == n
        assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(ws - 1))


def _worker(rank, world, port, o, p, e, sd, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        start, count = shard_chains(o.shape[0], world, rank)
        ol, pl, el = (torch.as_tensor(x[start:start + count]) for x in (o, p, e))
        mean, var, n = global_energy(el)
        jac = gq.SlicedJacobian(ol, pl, sd, gq.SliceOrdering())
        S, m, n2 = parameter_space_qgt(jac)
        go, gp = gather_jacobian(ol, pl)
        if rank == 0:
            out.put((float(mean), float(var), n, S.numpy(), go.numpy(), gp.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_one_process():
    shape, D, T, om, o, p, e = _data(50, 9)
    sd = oracle.sliced_dims(om)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, o, p, e, sd, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    mean, var, n, S, go, gp = res
    assert n == 50 and abs(mean - e.mean()) < 1e-12 and abs(var - e.var()) < 1e-12
    ref = osr.to_dense(osr.SlicedJacobian(o, p, sd, osr.SliceOrdering()), osr.ParameterSpace())
    assert np.allclose(S, ref, rtol=1e-10, atol=1e-12)
    assert np.array_equal(go, o) and np.array_equal(gp, p)


def _tdvp_driver(lib, group=None, integrator=None):
    from vmc_gb300 import PEPS, ZipUp
    from vmc_gb300.drivers import Euler, ImaginaryTimeUnit, TDVPDriver
    from vmc_gb300.operators import transverse_field_ising
    from vmc_gb300.preconditioners import SRPreconditioner
    from tests.helpers import uniform_init_tensors

    shape, D = (2, 3), 2
    model = PEPS(shape=shape, bond_dim=D, contraction_strategy=ZipUp(4), tensors=uniform_init_tensors(shape, D, seed=3),
                 device="cpu", lib=lib)
    # 5 chains over 2 ranks (3 + 2), 16 samples of 4 sweeps per chain (20 drawn, 16 kept)
    return TDVPDriver(model, transverse_field_ising(shape), dt=0.01, time_unit=ImaginaryTimeUnit(),
                      integrator=integrator or Euler(),
                      preconditioner=SRPreconditioner(space=gq.SampleSpace(), diag_shift=1e-2), n_samples=16,
                      n_chains=5, sampler_key=5, process_group=group)


def _tdvp_worker(rank, world, port, lib_path, out):
    from vmc_gb300 import _abi
    from vmc_gb300.drivers import RK4

    torch.set_num_threads(1)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        drv = _tdvp_driver(_abi.bind(lib_path), dist.group.WORLD, RK4())
        drv.run(0.02)
        out.put((rank, drv.model.packed().numpy().copy(), float(drv.energy["mean"]),
                 drv._sampler_configuration.numpy().copy()))
    finally:
        dist.destroy_process_group()


def test_sharded_tdvp_driver_equals_one_process(emu_lib):
    """TDVPDriver over 2 gloo ranks (uneven shards of 3 + 2 chains, two RK4 steps): both ranks end with the
    parameters and energy of the one-process run, bit for bit, and each holds its shard's configurations."""
    from tests.conftest import build_emulation_library
    from vmc_gb300.drivers import RK4

    n_threads = torch.get_num_threads()
    torch.set_num_threads(1)
    try:
        ref = _tdvp_driver(emu_lib, None, RK4())
        ref.run(0.02)
    finally:
        torch.set_num_threads(n_threads)
    theta = ref.model.packed().numpy()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + ((os.getpid() + 7) % 2000)
    procs = [ctx.Process(target=_tdvp_worker, args=(r, 2, port, str(build_emulation_library()), q))
             for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted([q.get(timeout=300) for _ in range(2)], key=lambda r: r[0])
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for rank, th, e, cfg in res:
        assert np.array_equal(th, theta), rank
        assert e == float(ref.energy["mean"])
    cfg_all = np.concatenate([r[3] for r in res])
    assert np.array_equal(cfg_all, ref._sampler_configuration.numpy())
