"""Population solvers driven by the batched fast-path statistic.

differential_evolution follows the reference's Differential Evolution fit
(solvers/diff_evoln_fit.cpp:104-160, solvers/DESolver.cpp:96-300):

* strategy rand-to-best/1 with exponential crossover
  (DESolver.cpp:357-374): starting at a random parameter, consecutive
  parameters take x + F (best - x) + F (x_r1 - x_r2) while a uniform draw
  stays below CR; F = 0.7, CR = 1.0;
* 8 members per free parameter; fixed parameters get lower = upper = value;
  every free parameter needs finite limits (diff_evoln_fit.cpp:118-142);
* initial members uniform in the limits, or Latin-hypercube samples
  (DESolver.cpp:114-151);
* a trial value outside its limits is redrawn uniformly between the limit and
  the member's current value (DESolver.cpp:229-236);
* convergence (DESolver.cpp:262-292): every 10 generations the relative change
  of the best energy since the previous check; from generation 40 on the fit
  has converged once the last three changes are all below ftol; at most 600
  generations.

Two things differ, both deliberately.  Each generation is synchronous: all
trial vectors are formed from the population as it stood at the start of the
generation and evaluated together in one batched GPU call
(imfit_BatchFitStatisticAndGradient, statistics only), whereas the reference
replaces members and the best vector in place while the generation runs.
And the initial population is evaluated once before generation 0, where the
reference starts every member at energy 1e20 with an all-zero best vector.
The trajectories therefore differ from the reference's; the optimum and the
convergence test do not.
"""
import numpy as np

MAX_DE_GENERATIONS = 600
POP_SIZE_PER_PARAMETER = 8


def _other_two(rng, NP):
    """Per member i, two distinct indices r1, r2 that differ from i."""
    i = np.arange(NP)
    r1 = (i + 1 + rng.integers(0, NP - 1, NP)) % NP
    a, b = np.minimum(i, r1), np.maximum(i, r1)
    r2 = rng.integers(0, NP - 2, NP)
    r2 = r2 + (r2 >= a)
    r2 = r2 + (r2 >= b)
    return r1, r2


def differential_evolution(model, x0, lower, upper, fixed=None, F=0.7, CR=1.0,
                           pop_per_param=POP_SIZE_PER_PARAMETER, max_generations=MAX_DE_GENERATIONS,
                           ftol=1e-8, seed=0, latin_hypercube=False):
    """Minimise model's fit statistic within [lower, upper].

    model needs batch_statistic_and_gradient(P, want_grad=False) -> statistics
    of the rows of P, and get_fit_statistic(x).  Returns a dict: params (the
    best vector), statistic (get_fit_statistic at it), generations, converged,
    population, batched_calls."""
    rng = np.random.default_rng(seed)
    x0 = np.asarray(x0, dtype=float)
    n = x0.size
    fixed = np.zeros(n, dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
    lo = np.where(fixed, x0, np.asarray(lower, dtype=float))
    hi = np.where(fixed, x0, np.asarray(upper, dtype=float))
    if np.any(~np.isfinite(lo)) or np.any(~np.isfinite(hi)) or np.any(lo > hi):
        raise ValueError("differential evolution needs finite limits lower <= upper for every free parameter")
    n_free = int(np.sum(~fixed))
    NP = pop_per_param * n_free
    if NP < 4:
        raise ValueError("differential evolution needs at least 4 population members")

    if latin_hypercube:
        perm = np.argsort(rng.random((n, NP)), axis=1).T  # [member, parameter] stratum index
        pop = lo + (perm + rng.random((NP, n))) * (hi - lo) / NP
    else:
        pop = lo + rng.random((NP, n)) * (hi - lo)
    energy = np.asarray(model.batch_statistic_and_gradient(pop, want_grad=False), dtype=float)
    calls = 1
    best = int(np.argmin(energy))

    deltas = [100.0, 100.0, 100.0]
    last_best = energy[best]
    converged = False
    generation = 0
    while generation < max_generations:
        r1, r2 = _other_two(rng, NP)
        mutant = pop + F * (pop[best] - pop) + F * (pop[r1] - pop[r2])
        # exponential crossover: L consecutive parameters from a random start
        start = (rng.random(NP) * n).astype(int)
        draws = rng.random((NP, n)) < CR
        L = np.where(draws.all(axis=1), n, np.argmin(draws, axis=1))
        offset = (np.arange(n)[None, :] - start[:, None]) % n
        take = offset < L[:, None]
        trial = np.where(take, mutant, pop)
        below, above = trial < lo, trial > hi
        u = rng.random((NP, n))
        trial = np.where(below, lo + u * (pop - lo), trial)
        trial = np.where(above, hi - u * (hi - pop), trial)
        e = np.asarray(model.batch_statistic_and_gradient(trial, want_grad=False), dtype=float)
        calls += 1
        better = e < energy
        pop[better] = trial[better]
        energy[better] = e[better]
        best = int(np.argmin(energy))

        if generation % 10 == 0:
            d = abs(1.0 - last_best / energy[best])
            if generation == 20:
                deltas[0] = d
            elif generation == 30:
                deltas = [d, deltas[0], deltas[2]]
            elif generation >= 40:
                deltas = [d, deltas[0], deltas[1]]
                if all(v < ftol for v in deltas):
                    converged = True
                    break
            last_best = energy[best]
        generation += 1
    xb = pop[best].copy()
    return dict(params=xb, statistic=model.get_fit_statistic(xb), generations=generation,
                converged=converged, population=NP, batched_calls=calls, fast_statistic=float(energy[best]))


# --------------------------------------------------------------------------
# Bootstrap resampling errors (core/bootstrap_errors.cpp:86-330,
# core/statistics.cpp:54-100).  All refits of a chunk run at once through
# imfit_BootstrapFitBatch; the samples are the same MT19937 index draws as the
# reference's sequential iterations, in the same order.

ONESIGMA_LOWER, ONESIGMA_UPPER = 0.1585, 0.8415


def _round_half_away(x):
    return int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5))


def standard_deviation(v):
    """statistics.cpp:54-72: sample standard deviation (n - 1)."""
    v = np.asarray(v, dtype=float)
    s = float(np.sum((v - np.mean(v)) ** 2))
    return float(np.sqrt(s / (v.size - 1))) if s >= 0 else 0.0


def confidence_interval(v):
    """statistics.cpp:84-100: the 68.3% interval from the sorted values at
    indices round(0.1585 n) - 1 and round(0.8415 n), clamped to the range."""
    v = np.sort(np.asarray(v, dtype=float))
    n = v.size
    lo = max(_round_half_away(ONESIGMA_LOWER * n) - 1, 0)
    hi = min(_round_half_away(ONESIGMA_UPPER * n), n - 1)
    return float(v[lo]), float(v[hi])


def bootstrap_errors(model, bestfit, n_iterations, seed, fixed=None, lower=None, upper=None, ftol=1e-8,
                     max_iter=0, chunk=64):
    """Bootstrap refits of model (chi^2 or Poisson-MLR) from bestfit; returns
    (params of the successful iterations [n_ok x nParams], statuses).  The
    reference seeds MT19937 with seed, draws one sample in UseBootstrap and
    then one per iteration (bootstrap_errors.cpp:171-215); so does this."""
    if seed <= 0:
        raise ValueError("give a positive seed (the reference seeds from the clock otherwise)")
    model.use_bootstrap(int(seed))
    out, statuses = [], []
    done = 0
    while done < n_iterations:
        k = min(chunk, n_iterations - done)
        r = model.bootstrap_fit_batch(k, bestfit, fixed=fixed, lower=lower, upper=upper, ftol=ftol,
                                      max_iter=max_iter)
        ok = r["status"] > 0
        out.append(r["params"][ok])
        statuses.append(r["status"])
        done += k
    return np.concatenate(out) if out else np.empty((0, len(bestfit))), np.concatenate(statuses)


def bootstrap_summary(bestfit, samples, names, fixed=None):
    """Lines of PrintBootstrapSummary (bootstrap_errors.cpp:339-369)."""
    samples = np.asarray(samples, dtype=float)
    n = samples.shape[0]
    fixed = np.zeros(len(bestfit), dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
    lines = ["", f"Statistics for parameter values from bootstrap resampling ({n} successful iterations):",
             "Best-fit\t\t Bootstrap      [68% conf.int., half-width]; (mean +/- standard deviation)"]
    for i, name in enumerate(names):
        if fixed[i]:
            lines.append(f"{name} = {bestfit[i]:g}     [fixed parameter]")
            continue
        lo, hi = confidence_interval(samples[:, i])
        sd = standard_deviation(samples[:, i])
        lines.append(f"{name} = {bestfit[i]:g}  +{hi - bestfit[i]:g}, -{bestfit[i] - lo:g}    "
                     f"[{lo:g} -- {hi:g}, {(hi - lo) / 2.0:g}];  ({np.mean(samples[:, i]):g} +/- {sd:g})")
    return lines


def bootstrap_file_lines(functions, param_names, n_params, samples, n_iterations):
    """The --save-bootstrap file (bootstrap_errors.cpp:111-114 and
    ModelObject::GetParamHeader / PrintModelParamsHorizontalString,
    core/model_object.cpp:1941-2033): functions = [(name, starts_new_set)],
    param_names = all parameter names in order, n_params = {name: count}."""
    header = "# "
    j, n_set = 0, 0
    for fi, (fname, new_set) in enumerate(functions):
        if new_set or fi == 0:
            n_set += 1
            header += f"X0_{n_set}\t\tY0_{n_set}\t\t"
            j += 2
        for _ in range(n_params[fname]):
            header += f"{param_names[j]}_{fi + 1}\t"
            j += 1
    lines = ["#", f"# Bootstrap resampling output ({n_iterations} iterations requested):", header]
    lines += ["\t".join(format(float(v), "#.10g") for v in row) for row in np.atleast_2d(samples)]
    return lines


# --------------------------------------------------------------------------
# DREAM Markov-chain Monte Carlo (cdream/dream.cpp:66-505 as imfit-mcmc sets
# it up, core/mcmc_main.cpp:360-440): differential-evolution proposals from
# delta chain pairs with randomised crossover (nCR = 3 values, their
# probabilities adapted during burn-in), Metropolis acceptance on
# log L = -statistic / 2, outlier chains moved to the best chain, and the
# Gelman-Rubin test on the second half of the post-burn-in samples.  The
# reference already forms every chain's proposal before evaluating any of
# them; here those evaluations are one batched GPU call per generation.
# Re-evaluating the previous states during burn-in (recalcLik + inBurnIn in
# dream.cpp:290-300) returns the same deterministic values and is skipped.
# The random stream is numpy's, not GSL's: chains are statistically, not
# bitwise, the reference's.

def _gsl_quantile_sorted(v, f):
    """gsl_stats_quantile_from_sorted_data: linear interpolation at (n-1) f."""
    delta = (len(v) - 1) * f
    lo = int(np.floor(delta))
    frac = delta - lo
    if lo + 1 < len(v):
        return (1.0 - frac) * v[lo] + frac * v[lo + 1]
    return v[lo]


def gelman_rubin(samples):
    """cdream/gelman_rubin.cpp with adjustDF = 0: samples [n][chains][vars];
    returns sqrt(Rhat) per variable (1 where the within-chain variance is 0)."""
    n, m = samples.shape[0], samples.shape[1]
    means = samples.mean(axis=0)                       # [chains][vars]
    W = samples.var(axis=0, ddof=1).mean(axis=0)       # mean within-chain variance
    Bdivn = means.var(axis=0, ddof=1)                  # variance of the chain means
    sigma2 = (n - 1.0) / n * W + Bdivn
    Vhat = sigma2 + Bdivn / m
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(W > 0.0, np.sqrt(Vhat / W), 1.0)
    return r


def dream(model, x0, lower, upper, fixed=None, n_chains=None, max_generations=100000, burn_in=5000,
          gelman_evals=5000, scale_reduction=1.01, noise=0.01, bstar=1.0e-6, n_cr=3, loop_steps=10,
          collapse_outliers=True, reenter_burnin=0.2, seed=0, callback=None):
    """DREAM on model's batched statistic (log L = -S/2).  Defaults are
    imfit-mcmc's (options_mcmc.h:72-79, dream_pars.cpp:8-45): n_chains = free
    parameters, 100000 generations at most, 5000 burn-in, a Gelman-Rubin check
    every gelman_evals generations (in loop_steps units) after burn-in,
    R-hat limit 1.01, noise b = 0.01, b* = 1e-6, deltaMax = (nfree - 1) / 2.
    callback(t, states[nChains][n], liks, in_burn_in, pCR, accept) is called
    after every generation (the chain files' rows).  Returns a dict with the
    chains [generations][chains][n], their log-likelihoods, burn-in flags and
    the convergence state."""
    rng = np.random.default_rng(seed)
    x0 = np.asarray(x0, dtype=float)
    nv = x0.size
    lock = np.zeros(nv, dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
    lo = np.where(lock, x0, np.asarray(lower, dtype=float))
    hi = np.where(lock, x0, np.asarray(upper, dtype=float))
    if np.any(~np.isfinite(lo[~lock])) or np.any(~np.isfinite(hi[~lock])):
        raise ValueError("MCMC needs finite limits for every free parameter")
    nfree = int(np.sum(~lock))
    nC = nfree if not n_chains or n_chains <= 0 else int(n_chains)
    if nC < 3:
        raise ValueError("DREAM needs at least 3 chains")
    delta_max = (nfree - 1) // 2
    gelman_loops = max(1, int(gelman_evals / 10))  # mcmc_main.cpp:412
    free = np.where(~lock)[0]

    def loglik(P, need):
        out = np.full(P.shape[0], -np.inf)
        if np.any(need):
            out[need] = -0.5 * np.asarray(model.batch_statistic_and_gradient(P[need], want_grad=False))
        return out

    # Latin-hypercube start (dream_initialize.cpp:18-62)
    perm = np.argsort(rng.random((nv, nC)), axis=1)  # samples(j, i)
    state0 = np.empty((nC, nv))
    for i in range(nC):
        for j in range(nv):
            if lock[j]:
                state0[i, j] = lo[j]
            else:
                v = lo[j] + perm[j, i] * (hi[j] - lo[j]) / nC + (hi[j] - lo[j]) / nC * rng.random()
                state0[i, j] = min(max(v, lo[j]), hi[j])
    states = [state0]
    liks = [loglik(state0, np.ones(nC, dtype=bool))]
    flags = [1 if burn_in > 0 else 0]
    in_burn = burn_in > 0
    burn_start = 0
    pCR = np.full(n_cr, 1.0 / n_cr)
    delta_tot = np.ones(n_cr)
    total_steps = np.zeros(n_cr)
    L = np.zeros(n_cr)
    CRm = None
    gen_number = 0
    cur_run = 0
    converged = False
    n_evals = nC
    accepted_total = 0
    scale_red = np.full(nv, np.inf)
    if callback:
        callback(0, state0, liks[0], in_burn, pCR, np.ones(nC, dtype=int))
    t = 0
    for t in range(1, max_generations):
        cur = states[-1]
        lcur = liks[-1]
        if gen_number == 0:  # gen_CR.cpp: multinomial counts of the nCR values, shuffled
            L = rng.multinomial(nC * loop_steps, pCR).astype(float)
            flat = np.repeat(np.arange(1, n_cr + 1), L.astype(int))
            rng.shuffle(flat)
            CRm = flat.reshape(nC, loop_steps)
        prop = cur.copy()
        update_dim = np.full(nC, nfree)
        for i in range(nC):
            delta = int(rng.integers(1, delta_max + 1)) if delta_max > 1 else 1
            r1 = rng.integers(0, nC - 1, size=delta)
            r1 = r1 + (r1 >= i)
            r2 = rng.integers(0, nC - 1, size=delta)
            for a in range(delta):
                while nC > 2 and (r2[a] == r1[a] or r2[a] == i):
                    r2[a] = (r2[a] + 1) % nC
            e = noise * (2.0 * rng.random(nv) - 1.0)
            eps = rng.normal(0.0, bstar, nv)
            pair = np.zeros(nv)
            for a in range(delta):
                if r1[a] != r2[a]:
                    pair += cur[r1[a]] - cur[r2[a]]
            cross = CRm[i, gen_number] / n_cr
            upd = ~lock.copy()
            if cross < 1.0:
                drop = rng.random(nv) < 1.0 - cross
                upd &= ~drop
            update_dim[i] = int(np.sum(upd))
            if update_dim[i] > 0:
                gamma = 1.0 if (t > 1 and t % 5 == 0) else 2.38 / np.sqrt(2.0 * update_dim[i] * delta)
                prop[i, upd] = cur[i, upd] + (1.0 + e[upd]) * gamma * pair[upd] + eps[upd]
        inside = np.all((prop[:, free] >= lo[free]) & (prop[:, free] <= hi[free]), axis=1)
        need = (update_dim > 0) & inside
        lnew = loglik(prop, need)
        n_evals += int(np.sum(need))
        lnew[update_dim == 0] = lcur[update_dim == 0]
        u = rng.random(nC)
        accept = np.where(np.isneginf(lnew), 0,
                          np.where(lnew >= lcur, 1, (np.log(u) < lnew - lcur).astype(int)))
        new = np.where(accept[:, None] == 1, prop, cur)
        lnew = np.where(accept == 1, lnew, lcur)
        accepted_total += int(accept.sum())
        if in_burn:  # crossover adaptation (dream.cpp:338-357)
            sd = new.std(axis=0, ddof=1)
            for i in range(nC):
                if accept[i]:
                    ok = (~lock) & (sd > 0.0)
                    delta_tot[CRm[i, gen_number] - 1] += float(np.sum(((new[i, ok] - cur[i, ok]) / sd[ok]) ** 2))
        gen_number += 1
        if gen_number >= loop_steps:
            gen_number = 0
            if in_burn:
                dsum = float(delta_tot.sum())
                total_steps += L
                if dsum > 0.0:
                    pCR = (delta_tot / dsum) / total_steps
                    pCR = pCR / pCR.sum()
            if collapse_outliers and t < reenter_burnin * max_generations:
                t0 = t // 2
                past = np.array(liks[t0:t] if t > t0 else [lnew])
                meanlik = past.mean(axis=0)
                srt = np.sort(meanlik)
                q1, q3 = _gsl_quantile_sorted(srt, 0.25), _gsl_quantile_sorted(srt, 0.75)
                out = meanlik < q1 - 2.0 * (q3 - q1)
                best = int(np.argmax(meanlik))
                for i in np.where(out)[0]:
                    if i == best:
                        continue
                    new[i] = new[best]
                    lnew[i] = lnew[best]
                    if not in_burn and burn_in > 0:
                        burn_start, cur_run, in_burn = t, 0, True
            if not in_burn:
                cur_run += 1
                if cur_run >= gelman_loops:
                    first = burn_start + burn_in
                    t0 = (t + first) // 2
                    n = t - t0 - 1
                    if n > 1:
                        S = np.array(states[t0:t0 + n])
                        scale_red = gelman_rubin(S)
                        if np.all(scale_red[free] < scale_reduction):
                            converged = True  # the reference stops before recording generation t
                            break
                    cur_run = 0
            elif t >= burn_start + burn_in:
                in_burn = False
        states.append(new)
        liks.append(lnew)
        flags.append(1 if t < burn_start + burn_in else 0)
        if callback:
            callback(t, new, lnew, t < burn_start + burn_in, pCR, accept)
    return dict(chains=np.array(states), loglik=np.array(liks), burn_in=np.array(flags), converged=converged,
                generations=len(states), n_chains=nC, evaluations=n_evals, scale_reduction=scale_red,
                acceptance=accepted_total / max(1, nC * t), burn_in_end=burn_start + burn_in)


def chain_file_header(functions, param_names, n_params, n_cr=3):
    """Column-header line of an imfit-mcmc chain file (core/mcmc_main.cpp:421-428)."""
    head = bootstrap_file_lines(functions, param_names, n_params, np.empty((0, len(param_names))), 0)[2]
    head += "  likelihood  burn-in    "
    head += "".join(f"CR{i + 1}               " for i in range(n_cr - 1)) + f"CR{n_cr}        accept"
    return head


def chain_file_row(params, loglik, burn_in, pCR, accept):
    """One chain-file row (cdream/dream.cpp:458-468): the parameters as
    PrintModelParamsHorizontalString writes them, then log L, the burn-in flag,
    the crossover probabilities (scientific, 12 digits) and the acceptance."""
    row = "\t".join(format(float(v), "#.10g") for v in params)
    row += f" {loglik:.12e} {int(burn_in)}  " + "".join(f"{float(p):.12e} " for p in pCR) + f"{int(accept)}"
    return row


def nelder_mead(model, x0, lower, upper, fixed=None, ftol=1e-8, max_evals=None):
    """Nelder-Mead simplex on the FP64 statistic (GetFitStatistic), as
    solvers/nmsimplex_fit.cpp:160-210 sets NLopt's NLOPT_LN_NELDERMEAD up:
    relative and absolute f tolerance ftol, relative x tolerance ftol,
    10000 x nParams evaluations at most, box limits.  NLopt is not in this
    image: scipy's Nelder-Mead (Gao-Han adaptive coefficients off) stands in,
    so the path to the minimum differs from NLopt's while the minimum does not.
    Fixed parameters are held out of the simplex."""
    from scipy.optimize import minimize
    x0 = np.asarray(x0, dtype=float)
    n = x0.size
    fixed = np.zeros(n, dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
    free = np.where(~fixed)[0]
    lo = np.asarray(lower, dtype=float)
    hi = np.asarray(upper, dtype=float)
    count = [0]

    def f(z):
        x = x0.copy()
        x[free] = z
        count[0] += 1
        return model.get_fit_statistic(x)

    bounds = [(lo[j] if np.isfinite(lo[j]) else None, hi[j] if np.isfinite(hi[j]) else None) for j in free]
    res = minimize(f, x0[free], method="Nelder-Mead", bounds=bounds,
                   options=dict(xatol=ftol * max(1.0, float(np.max(np.abs(x0[free])))), fatol=ftol,
                                maxfev=max_evals or 10000 * n, adaptive=False))
    x = x0.copy()
    x[free] = res.x
    return dict(params=x, statistic=model.get_fit_statistic(x), evaluations=count[0], converged=bool(res.success))
