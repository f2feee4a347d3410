"""Adjoint gradients of batched closed adiabatic reactor integrations with respect to the Arrhenius parameters.

Outputs per reactor, after integrating to t_end with the reference's adaptive ESDIRK64 (defaults of
HomogeneousReactor.integrate, reactors.py:429-611):
  * T_end: the temperature at t_end;
  * tau_s: a smoothed ignition delay, the ESDIRK64 quadrature of the time spent below T0 + 400 K,
        tau_s = sum_n h_n sum_s b_s g(T(Y_ns)),   g(T) = 1 - 1 / (1 + exp(-(T - T0 - 400 K) / 20 K)),
    which tends to the ignition delay as the 20 K width goes to zero.
Parameters theta: ln A_r and E_a,r (J/kmol) of every reaction, the forward or for falloff reactions the
high-pressure Arrhenius coefficients, reported in the mechanism file's reaction order.

Method: the discrete adjoint of the recorded ESDIRK64 step sequence (the gradient of the computed outputs for the
accepted step sizes, with stage equations solved exactly; the reference computes no sensitivities). The forward
run records every accepted step's size and six stage values in HBM (``sf_integrate_record_batch``), the
per-step checkpoint. Backwards through the steps, all active reactors at once: stage Jacobians J_s and
right-hand sides at the recorded stages (one batched launch), the transposed stage systems
(I - h gamma J_s^T) w_s = c_s with c_s = h b_s lam' + h sum_{l>s} a_ls Ybar_l + h gamma q_s (batched LU and
solves), Ybar_s = J_s^T w_s + q_s, lam_n = lam' + sum_s Ybar_s, where lam' is lam_{n+1} with the entries the
post-step clamp of negative values zeroed and q_s the quadrature term of tau_s; and the parameter adjoint
theta_bar += sum_s w_s^T df/dtheta(Y_s) (``sf_rate_param_adjoint_batch``). ``IgnitionOutputs`` exposes the same
computation as a torch.autograd.Function of theta.
"""

import copy
import ctypes as C

import numpy as np

from . import _native as N
from ._desc import reactor_params
from .linalg import NewtonSystems
from .reactors import BatchIntegrator

GAMMA = 0.25
_A = np.array([[0., 0., 0., 0., 0., 0.],
               [0.25, GAMMA, 0., 0., 0., 0.],
               [8611. / 62500., -1743. / 31250., GAMMA, 0., 0., 0.],
               [5012029. / 34652500., -654441. / 2922500., 174375. / 388108., GAMMA, 0., 0.],
               [15267082809. / 155376265600., -71443401. / 120774400., 730878875. / 902184768.,
                2285395. / 8070912., GAMMA, 0.],
               [82889. / 524892., 0., 15625. / 83664., 69875. / 102672., -2260. / 8211., GAMMA]])
_B = _A[5].copy()
DT_IGN = 400.
WIDTH = 20.
OUTPUT_KINDS = {'T_end': 0, 'tau_s': 1}  # sf_adjoint_output


def _torch():
    import torch
    return torch


def nominal_parameters(mech):
    """theta [n_reactions, 2] = (ln A, E_a in J/kmol) in the mechanism file's reaction order."""
    rx = mech.mech_data['reactions']
    th = np.zeros((len(rx), 2))
    yi = mech.reaction_yaml_index
    for r, t in enumerate(rx):
        th[yi[r]] = (np.log(t[4]), t[6])
    return th


def mechanism_with_parameters(mech, theta):
    """A copy of the mechanism whose reactions carry A = exp(theta[:, 0]) and E_a = theta[:, 1] (file order)."""
    from .mechanism import ChemicalMechanismSpec
    theta = np.asarray(theta, dtype=np.float64)
    md = copy.deepcopy(mech.mech_data)
    yi = mech.reaction_yaml_index
    for r in range(len(md['reactions'])):
        t = list(md['reactions'][r])
        t[4] = float(np.exp(theta[yi[r], 0]))
        t[6] = float(theta[yi[r], 1])
        md['reactions'][r] = tuple(t)
    out = ChemicalMechanismSpec(mech_data=md)
    out._reaction_yaml_index = list(yi)
    return out


class Trajectory:
    """A recorded batched integration (device tensors)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


class ReactorAdjoint:
    def __init__(self, mech, configuration='isobaric', pressure=101325.):
        self.mech = mech
        self.g = mech.griffon
        self.configuration = configuration
        self.pressure = pressure
        self.params = reactor_params(configuration, 'adiabatic', pressure=pressure)
        self.ns = mech.n_species
        self.neq = self.ns if configuration == 'isobaric' else self.ns + 1
        self.tix = 0 if configuration == 'isobaric' else 1
        self.nr = len(mech.mech_data['reactions'])
        self.integrator = BatchIntegrator(mech, configuration, pressure=pressure)

    # ------------------------------------------------------------------------------------------------- forward
    def forward(self, q0, pressures=None, t_end=5.e-3, capacity=None, **controls):
        """Integrate every row of q0 to t_end, recording the steps. The record starts at `capacity` steps per
        reactor (None: BatchIntegrator.default_record_capacity, up to 1024 within a quarter of the free device
        memory) and grows for the reactors that run out of it, which alone are integrated again."""
        torch = _torch()
        q0 = self.g._dev(q0)
        n = q0.shape[0]
        if pressures is None:
            pressures = torch.full((n,), float(self.pressure), dtype=torch.float64, device=q0.device)
        pressures = self.g._dev(pressures)
        ip = self.integrator.controls(stop_at_time=t_end, **controls)
        out, rec = self.integrator.record(q0, pressures, ip, capacity or self.integrator.default_record_capacity(n))
        capacity = rec.shape[1]
        steps = out['counts'][:, 0].long()
        T0 = q0[:, self.tix].clone()
        # smoothed ignition delay by the ESDIRK64 quadrature of the recorded stages
        Bt = torch.tensor(_B, dtype=torch.float64, device=q0.device)
        h = rec[:, :, 1]
        Ts = rec[:, :, 2:].view(n, capacity, 6, self.neq)[..., self.tix]
        # slots past a reactor's last step hold whatever the buffer held: select, do not multiply by zero
        valid = torch.arange(capacity, device=q0.device)[None, :] < steps[:, None]
        g = 1. - torch.sigmoid((Ts - T0[:, None, None] - DT_IGN) / WIDTH)
        contrib = h * (g * Bt).sum(-1)
        tau = torch.where(valid, contrib, torch.zeros_like(contrib)).sum(1)
        return Trajectory(q0=q0, pressures=pressures, rec=rec, steps=steps, status=out['status'], q_end=out['q'],
                          t_end=out['t'], T0=T0, T_end=out['q'][:, self.tix].clone(), tau_s=tau,
                          counts=out['counts'])

    # ------------------------------------------------------------------------------------------------ backward
    def backward(self, traj, outputs=('T_end', 'tau_s')):
        """Gradients of the outputs of every reactor, by the native backward sweep (sf_adjoint_batch). Returns
        dict(theta=[n, n_out, n_reactions, 2] (d/d ln A, d/d E_a) in file order, q0=[n, n_out, neq] (gradients with
        respect to the initial state))."""
        torch = _torch()
        kinds = []
        for name in outputs:
            if name not in OUTPUT_KINDS:
                raise ValueError(f'unknown output {name}')
            kinds.append(OUTPUT_KINDS[name])
        n, neq, nr, O = traj.q0.shape[0], self.neq, self.nr, len(outputs)
        dev = traj.q0.device
        theta_int = torch.empty((n, O, 2 * nr), dtype=torch.float64, device=dev)
        q0g = torch.empty((n, O, neq), dtype=torch.float64, device=dev)
        L = N.load()
        if n:
            nb = int(L.sf_adjoint_workspace_size(self.g.handle, C.byref(self.params), n, O))
            ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=dev)
            kk = (C.c_int * O)(*kinds)
            T0 = traj.T0.contiguous()
            N.check(L.sf_adjoint_batch(self.g.handle, C.byref(self.params), n, N.ptr(traj.rec), traj.rec.shape[1],
                                       N.ptr(traj.counts), N.ptr(traj.pressures), N.ptr(T0), O,
                                       C.cast(kk, C.c_void_p), N.ptr(theta_int), N.ptr(q0g), N.ptr(ws), nb,
                                       N.stream_handle()))
            del ws
        G = theta_int.view(n, O, nr, 2)
        yi = torch.as_tensor(self.mech.reaction_yaml_index, device=dev)
        theta = torch.empty_like(G)
        theta[:, :, yi] = G
        return dict(theta=theta, q0=q0g)

    def backward_host(self, traj, outputs=('T_end', 'tau_s')):
        """The backward sweep of ``backward`` with its step loop in Python over torch operations and the batched
        primitives (chemistry Jacobians, Newton LU/solves, the parameter adjoint): the same recursion, kept to check
        the native sweep against."""
        torch = _torch()
        dev = traj.q0.device
        n, neq, tix, nr = traj.q0.shape[0], self.neq, self.tix, self.nr
        O = len(outputs)
        lam = torch.zeros((n, O, neq), dtype=torch.float64, device=dev)
        for o, name in enumerate(outputs):
            if name == 'T_end':
                lam[:, o, tix] = 1.
            elif name != 'tau_s':
                raise ValueError(f'unknown output {name}')
        quad = torch.tensor([1. if name == 'tau_s' else 0. for name in outputs], dtype=torch.float64, device=dev)
        grad = torch.zeros((n * O, 2 * nr), dtype=torch.float64, device=dev)
        A = torch.tensor(_A, dtype=torch.float64, device=dev)
        Bt = torch.tensor(_B, dtype=torch.float64, device=dev)
        steps = traj.steps
        nmax = int(steps.max().item()) if n else 0
        L = N.load()
        for m in range(nmax):
            act = torch.nonzero(steps > m).squeeze(1)
            na = act.numel()
            idx = steps[act] - 1 - m
            row = traj.rec[act, idx]                                   # [na, 2 + 6 neq]
            h = row[:, 1]
            Y = row[:, 2:].reshape(na, 6, neq)
            pres = traj.pressures[act]
            k, J = self.g.reactor_jac_batch(self.params, Y.reshape(na * 6, neq), 0,
                                            pressures=pres.repeat_interleave(6))
            k = k.view(na, 6, neq)
            JT = J.view(na, 6, neq, neq)                               # row-major view of J^T
            # the post-step clamp of negative entries has zero derivative where it acted
            v = Y[:, 0] + h[:, None] * torch.einsum('s,asn->an', Bt, k)
            lamp = lam[act] * (v >= 0.).double()[:, None, :]
            # quadrature terms of tau_s: q_s = h b_s g'(T_s) e_T
            Ts = Y[:, :, tix]
            sg = torch.sigmoid((Ts - traj.T0[act][:, None] - DT_IGN) / WIDTH)
            dg = -sg * (1. - sg) / WIDTH
            qd = torch.zeros((na, O, 6, neq), dtype=torch.float64, device=dev)
            qd[:, :, :, tix] = (h[:, None] * Bt[None, :] * dg)[:, None, :] * quad[None, :, None]
            # factors of the transposed implicit stage systems, stage-major: system (s-1)*na + a
            JTcm = JT[:, 1:].transpose(-1, -2).transpose(0, 1).contiguous().view(5 * na, neq * neq)
            ghs = (h * GAMMA).repeat(5)
            fac = NewtonSystems(5 * na, neq, 0, device=dev).factor(JTcm, ghs)
            W = torch.zeros((na, O, 6, neq), dtype=torch.float64, device=dev)
            Ybar = torch.zeros((na, O, 6, neq), dtype=torch.float64, device=dev)
            for s in range(5, -1, -1):
                c = h[:, None, None] * Bt[s] * lamp
                for l in range(s + 1, 6):
                    if A[l, s] != 0.:
                        c = c + h[:, None, None] * A[l, s] * Ybar[:, :, l]
                if s >= 1:
                    c = c + (h * GAMMA)[:, None, None] * qd[:, :, s]
                    w = torch.empty_like(c)
                    for o in range(O):
                        # (h gamma J^T - I) w = -c
                        w[:, o] = fac.solve((-c[:, o]).contiguous(), start=(s - 1) * na, count=na)
                else:
                    w = c
                W[:, :, s] = w
                Ybar[:, :, s] = torch.einsum('aij,aoj->aoi', JT[:, s], w) + qd[:, :, s]
            del fac
            lam[act] = lamp + Ybar.sum(2)
            # parameter adjoint over the six stages of every (reactor, output) item
            q_items = Y[:, None].expand(na, O, 6, neq).reshape(na * O, 6, neq).contiguous()
            w_items = W.reshape(na * O, 6, neq).contiguous()
            p_items = pres.repeat_interleave(O).contiguous()
            tmp = torch.zeros((na * O, 2 * nr), dtype=torch.float64, device=dev)
            N.check(L.sf_rate_param_adjoint_batch(self.g.handle, C.byref(self.params), na * O, 6, N.ptr(q_items),
                                                  N.ptr(p_items), N.ptr(w_items), N.ptr(tmp), N.stream_handle()))
            rows = (act[:, None] * O + torch.arange(O, device=dev)[None, :]).reshape(-1)
            grad.index_add_(0, rows, tmp)
        G = grad.view(n, O, nr, 2)
        yi = torch.as_tensor(self.mech.reaction_yaml_index, device=dev)
        theta = torch.empty_like(G)
        theta[:, :, yi] = G
        return dict(theta=theta, q0=lam)


def _make_function():
    torch = _torch()

    class IgnitionOutputs(torch.autograd.Function):
        """(T_end, tau_s) [n, 2] of closed adiabatic reactors as a function of theta [n_reactions, 2]
        (ln A, E_a in J/kmol, file order); backward runs the batched discrete adjoint."""

        @staticmethod
        def forward(ctx, theta, mech, q0, pressures, t_end, configuration, pressure):
            th = theta.detach().cpu().numpy()
            m = mech if np.array_equal(th, nominal_parameters(mech)) else mechanism_with_parameters(mech, th)
            adj = ReactorAdjoint(m, configuration, pressure)
            traj = adj.forward(q0, pressures, t_end)
            ctx.adj, ctx.traj, ctx.theta_device = adj, traj, theta.device
            return torch.stack([traj.T_end, traj.tau_s], dim=1)

        @staticmethod
        def backward(ctx, grad_out):
            G = ctx.adj.backward(ctx.traj)['theta']  # [n, 2, nr, 2]
            ctx.per_reactor = G
            gth = (grad_out.to(G.device)[:, :, None, None] * G).sum((0, 1)).to(ctx.theta_device)
            return gth, None, None, None, None, None, None

    return IgnitionOutputs


_FN = None


def ignition_outputs(theta, mech, q0, pressures=None, t_end=5.e-3, configuration='isobaric', pressure=101325.):
    """Differentiable (T_end, tau_s) [n, 2] with respect to theta (a CUDA or CPU FP64 tensor [n_reactions, 2])."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(theta, mech, q0, pressures, t_end, configuration, pressure)
