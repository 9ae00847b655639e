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
