"""Alpert hybrid Gauss-trapezoidal correction for log-singular kernels on a
closed periodic boundary component (CFIE_alpert; cfie_alpert.jl:56-232,
371-431, 724-789; rules alpert_table.jl:46-89).

On the periodic midpoint grid u_j = (j - 1/2)/N the self block of a smooth
closed component is the trapezoid rule with the near band |j - i| < a
removed, plus 2j correction nodes per target at u_i +/- xi_p/N with weights
h w_p whose kernel values are spread onto the grid by Lagrange interpolation
over ninterp = order + 3 nodes. This module builds, on the host, the
per-target geometry of the correction nodes (the curve is known only here)
and the interpolation stencils; the device assembles the operator.

The rule table holds the published node/weight values of
B. K. Alpert, "Hybrid Gauss-trapezoidal quadrature rules", SIAM J. Sci.
Comput. 20 (1999) 1551-1584, for the log-singular end correction (the same
values as the reference, which parity requires).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * math.pi

# order: (a = near-band width, nodes x_p, weights w_p)
ALPERT_LOG_RULES = {
    2: (1, [1.591549430918953e-01], [5.0e-01]),
    3: (2, [1.150395811972836e-01, 9.365464527949632e-01], [3.913373788753340e-01, 1.108662621124666e+00]),
    4: (2, [2.379647284118974e-02, 2.935370741501914e-01, 1.023715124251890e+00],
        [8.795942675593887e-02, 4.989017152913699e-01, 9.131388579526912e-01]),
    5: (3, [2.339013027203800e-02, 2.854764931311984e-01, 1.005403327220700e+00, 1.994970303994294e+00],
        [8.609736556158105e-02, 4.847019685417959e-01, 9.152988869123725e-01, 1.013901778984250e+00]),
    6: (3, [4.004884194926570e-03, 7.745655373336686e-02, 3.972849993523248e-01, 1.075673352915104e+00,
            2.003796927111872e+00],
        [1.671879691147102e-02, 1.636958371447360e-01, 4.981856569770637e-01, 8.372266245578912e-01,
         9.841730844088381e-01]),
    8: (5, [6.531815708567918e-03, 9.086744584657729e-02, 3.967966533375878e-01, 1.027856640525646e+00,
            1.945288592909266e+00, 2.980147933889640e+00, 3.998861349951123e+00],
        [2.462194198995203e-02, 1.701315866854178e-01, 4.609256358650077e-01, 7.947291148621894e-01,
         1.008710414337933e+00, 1.036093649726216e+00, 1.004787656533285e+00]),
    10: (6, [1.175089381227308e-03, 1.877034129831289e-02, 9.686468391426860e-02, 3.004818668002884e-01,
             6.901331557173356e-01, 1.293695738083659e+00, 2.090187729798780e+00, 3.016719313149212e+00,
             4.001369747872486e+00, 5.000025661793423e+00],
         [4.560746882084207e-03, 3.810606322384757e-02, 1.293864997289512e-01, 2.884360381408835e-01,
          4.958111914344961e-01, 7.077154600594529e-01, 8.741924365285083e-01, 9.661361986515218e-01,
          9.957887866078700e-01, 9.998665787423845e-01]),
    12: (7, [1.674223682668368e-03, 2.441110095009738e-02, 1.153851297429517e-01, 3.345898490480388e-01,
             7.329740531807683e-01, 1.332305048525433e+00, 2.114358752325948e+00, 3.026084549655318e+00,
             4.003166301292590e+00, 5.000141170055870e+00, 6.000001002441859e+00],
         [6.364190780720557e-03, 4.723964143287529e-02, 1.450891158385963e-01, 3.021659470785897e-01,
          4.984270739715340e-01, 6.971213795176096e-01, 8.577295622757315e-01, 9.544136554351155e-01,
          9.919938052776484e-01, 9.994621875822987e-01, 9.999934408092805e-01]),
    14: (9, [9.305182368545380e-04, 1.373832458434617e-02, 6.630752760779359e-02, 1.979971397622003e-01,
             4.504313503816532e-01, 8.571888631101634e-01, 1.434505229617112e+00, 2.175177834137754e+00,
             3.047955068386372e+00, 4.004974906813428e+00, 4.998525901820967e+00, 5.999523015116678e+00,
             6.999963617883990e+00, 7.999999488130134e+00],
         [3.545060644780164e-03, 2.681514031576498e-02, 8.504092035093420e-02, 1.854526216643691e-01,
          3.251724374883192e-01, 4.911553747260108e-01, 6.622933417369036e-01, 8.137254578840510e-01,
          9.235595514944174e-01, 9.821609923744658e-01, 1.000047394596121e+00, 1.000909336693954e+00,
          1.000119534283784e+00, 1.000002835746089e+00]),
    16: (10, [8.371529832014113e-04, 1.239382725542637e-02, 6.009290785739468e-02, 1.805991249601928e-01,
              4.142832599028031e-01, 7.964747731112430e-01, 1.348993882467059e+00, 2.073471660264395e+00,
              2.947904939031494e+00, 3.928129252248612e+00, 4.957203086563112e+00, 5.986360113977494e+00,
              6.997957704791519e+00, 7.999888757524622e+00, 8.999998754306120e+00],
         [3.190919086626234e-03, 2.423621380426338e-02, 7.740135521653088e-02, 1.704889420286369e-01,
          3.029123478511309e-01, 4.652220834914617e-01, 6.401489637096768e-01, 8.051212946181061e-01,
          9.362411945698647e-01, 1.014359775369075e+00, 1.035167721053657e+00, 1.020308624984610e+00,
          1.004798397441514e+00, 1.000395017352309e+00, 1.000007149422537e+00]),
}


@dataclass
class AlpertRule:
    order: int
    a: int
    x: np.ndarray
    w: np.ndarray

    @property
    def j(self) -> int:
        return len(self.x)


def alpert_log_rule(order: int) -> AlpertRule:
    if order not in ALPERT_LOG_RULES:
        raise ValueError(f"unsupported Alpert order {order}; available: {sorted(ALPERT_LOG_RULES)}")
    a, x, w = ALPERT_LOG_RULES[order]
    return AlpertRule(order, a, np.asarray(x, float), np.asarray(w, float))


def lagrange_weights(xi: float, nodes: np.ndarray) -> np.ndarray:
    """l_j(xi) = prod_{l != j} (xi - x_l) / (x_j - x_l)."""
    nodes = np.asarray(nodes, float)
    w = np.empty(len(nodes))
    for j, xj in enumerate(nodes):
        others = np.delete(nodes, j)
        w[j] = np.prod(xi - others) / np.prod(xj - others)
    return w


def interp_offsets_weights(xi: float, ninterp: int):
    """Stencil of ninterp consecutive integer offsets around xi and its Lagrange weights."""
    j0 = math.floor(xi - ninterp / 2 + 1)
    offs = np.arange(j0, j0 + ninterp)
    return offs, lagrange_weights(xi, offs.astype(float))


@dataclass
class PeriodicCache:
    """Correction-node geometry of one component, arrays [p, i] (j x N)."""
    rp: np.ndarray
    rm: np.ndarray
    innp: np.ndarray
    innm: np.ndarray
    sp: np.ndarray
    sm: np.ndarray
    offp: np.ndarray  # [p, m]
    wtp: np.ndarray
    offm: np.ndarray
    wtm: np.ndarray
    ninterp: int


def _orientation_sign(ts: np.ndarray) -> int:
    if len(ts) < 2:
        return 1
    d = math.fmod(ts[1] - ts[0] + math.pi, TWO_PI)
    d = d + TWO_PI if d < 0 else d
    return 1 if d - math.pi >= 0 else -1


def periodic_cache(crv, pts, rule: AlpertRule, order: int) -> PeriodicCache:
    """_build_alpert_periodic_cache (cfie_alpert.jl:724-789) for one closed curve."""
    N = pts.n
    J = rule.j
    ninterp = order + 3
    sg = _orientation_sign(pts.ts)
    X, Y = pts.xy[:, 0], pts.xy[:, 1]
    u = pts.ts / TWO_PI
    out = {k: np.empty((J, N)) for k in ("rp", "rm", "innp", "innm", "sp", "sm")}
    offp = np.empty((J, ninterp), np.int64)
    offm = np.empty((J, ninterp), np.int64)
    wtp = np.empty((J, ninterp))
    wtm = np.empty((J, ninterp))
    eps = np.finfo(float).eps
    for p in range(J):
        xi = rule.x[p]
        offp[p], wtp[p] = interp_offsets_weights(xi, ninterp)
        offm[p], wtm[p] = interp_offsets_weights(-xi, ninterp)
        du = sg * xi / N
        for side, shift in (("p", du), ("m", -du)):
            us = np.mod(u + shift, 1.0)
            q = crv.curve(us)
            t = sg * crv.tangent(us) / TWO_PI
            dx, dy = X - q[:, 0], Y - q[:, 1]
            r2 = dx * dx + dy * dy
            ok = np.isfinite(r2) & (r2 > eps * eps)
            out["r" + side][p] = np.where(ok, np.sqrt(np.where(ok, r2, 1.0)), np.inf)
            out["inn" + side][p] = np.where(ok, t[:, 1] * dx - t[:, 0] * dy, 0.0)
            out["s" + side][p] = np.hypot(t[:, 0], t[:, 1])
    return PeriodicCache(out["rp"], out["rm"], out["innp"], out["innm"], out["sp"], out["sm"], offp, wtp, offm,
                         wtm, ninterp)
