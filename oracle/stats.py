"""Oracle (test infrastructure only): a plain-Python restatement of the
reference's statistics stage, used to check the C++ host adapter's binning,
jackknife and output (fk_mc_gb300/host/fk_mc/binning.hpp, jackknife.hpp,
data_save.hpp). Pinned against the binning and jackknife known answers of the
reference's own tests (test/binning_test.cpp, test/jackknife_test.cpp), kept in
tests/golden/reference_kats.json.

Each function follows the reference file and lines named in its docstring.
"""
import math


def binned(x, depth):
    """Bins of 2^depth consecutive samples by repeated pairwise averaging
    (include/fk_mc/binning.hpp:30-40 binned_iterator::dereference, :70-87
    calc_bin_size / find_bin_range: the incomplete tail is dropped)."""
    step = 1 << depth
    if step > len(x):
        raise ValueError(f"Can't bin with binning step({step})> container size ({len(x)})")
    level = [float(v) for v in x[:(len(x) // step) * step]]
    for _ in range(depth):
        level = [(level[2 * k] + level[2 * k + 1]) / 2. for k in range(len(level) // 2)]
    return level


def calc_stats(v):
    """(size, mean, variance with size-1, sqrt(variance/size)), summed left to
    right (include/fk_mc/binning.hpp:90-97)."""
    size = len(v)
    s = 0.0
    for y in v:
        s += y
    mean = s / size
    sq = 0.0
    for y in v:
        sq += (y - mean) * (y - mean)
    var = sq / (size - 1) if size > 1 else float("nan")
    return (size, mean, var, math.sqrt(var / size) if size > 1 else float("nan"))


def accumulate_binning(x, max_depth):
    """Statistics of depths 0..max_depth (include/fk_mc/binning.hpp:106-160)."""
    return [calc_stats(binned(x, d)) for d in range(max_depth + 1)]


def cor_length(rows):
    """0.5 (2^i var_i / var_0 - 1) (include/fk_mc/binning.hpp:168-176)."""
    return [0.5 * (2. ** i * r[2] / rows[0][2] - 1) for i, r in enumerate(rows)]


def estimate_bin(rows):
    """prog/data_save.hpp:108-122."""
    errors = [r[3] for r in rows]
    rel = 1.
    ind = len(errors) - 1
    f = True
    while f and ind > 0:
        cur = abs(errors[ind - 1] / errors[ind] - 1.)
        f = cur < 0.05 and cur < rel
        if f:
            rel = cur
            ind -= 1
    return ind


def jack(F, series, depth):
    """include/fk_mc/jackknife.hpp:47-80 (jackknife_adapter::jack) on series
    binned at `depth`."""
    x = [binned(s, depth) for s in series]
    size = len(x[0])
    means = [calc_stats(s)[1] for s in x]
    U0 = F(means)
    U = [F([(size * means[i] - x[i][j]) / (size - 1) for i in range(len(x))]) for j in range(size)]
    st = calc_stats(U)
    Ubar = st[1]
    avg = U0 - (size - 1) * (Ubar - U0)
    dU = (size - 1) * st[3]
    return (size, avg, dU * dU * size, dU)


def accumulate_jackknife(F, series, max_depth):
    return [jack(F, series, d) for d in range(max_depth + 1)]


FUNCS = {
    "mean": lambda x: x[0],
    "disp": lambda x: x[1] - x[0] * x[0],                 # prog/data_save.hxx:212
    "binder": lambda x: 1. - x[1] / 3. / x[0] / x[0],     # prog/data_save.hxx:229
}


def cv_function(beta, volume):
    """prog/data_save.hxx:187."""
    return lambda x: beta * beta * (x[1] - x[2] - x[0] * x[0]) / volume


def default_max_bin(n):
    """prog/data_save.hpp:90 (n = 0 gives 1, as the reference's clamp does)."""
    if n == 0:
        return 1
    v = math.log(n / 16) / math.log(2.) - 1
    return min(15, max(int(v), 1))


def save_all(obs, beta, volume, dos_npts=240, dos_width=6.0, dos_offset=0.05, measure_history=True,
             measure_ipr=False, measure_stiffness=False, wgrid_cond=(), max_bin=-1):
    """The quantities prog/data_save.hxx:32-95 saves, as a dict:
    binning[name] = rows, stats[name] = (depth, row), tables[name] = rows.
    obs: dict of lists (histories state-major)."""
    out = {"binning": {}, "stats": {}, "tables": {}}
    nmeas = len(obs.get("nfpi") or obs.get("energies") or [])
    mb = max_bin if max_bin >= 0 else default_max_bin(nmeas)

    def save_binning(rows, name):
        out["binning"][name] = [list(r) + [c] for r, c in zip(rows, cor_length(rows))]
        b = estimate_bin(rows)
        out["stats"][name] = (b, rows[b])

    e = obs.get("energies")
    if e:
        d2 = obs["d2energies"]
        save_binning(accumulate_binning(e[::-1], mb), "energy")
        save_binning(accumulate_binning(d2[::-1], mb), "d2energy")
        if obs.get("c_energies"):
            save_binning(accumulate_binning(obs["c_energies"][::-1], mb), "c_energy")
        e2 = [v * v for v in e]
        save_binning(accumulate_jackknife(cv_function(beta, volume), [e[::-1], e2[::-1], d2[::-1]], mb), "cv")
    nf0, nfpi = obs.get("nf0"), obs.get("nfpi")
    if nf0 and nfpi:   # prog/data_save.hxx:202-236
        nn0, nnpi = [v * v for v in nf0], [v * v for v in nfpi]
        n40, n4pi = [v * v * v * v for v in nf0], [v * v * v * v for v in nfpi]
        save_binning(accumulate_binning(nf0[::-1], mb), "nf_0")
        save_binning(accumulate_binning(nfpi[::-1], mb), "nf_pi")
        fs0 = accumulate_jackknife(FUNCS["disp"], [nf0, nn0], mb)
        save_binning(fs0, "fsusc_0")
        save_binning(accumulate_jackknife(FUNCS["disp"], [nfpi, nnpi], mb), "fsusc_pi")
        b = estimate_bin(fs0)
        out["stats"]["binder_0"] = (b, jack(FUNCS["binder"], [nn0, n40], b))
        out["stats"]["binder_pi"] = (b, jack(FUNCS["binder"], [nnpi, n4pi], b))
    grid = [-dos_width + 2. * dos_width * i / (1. * dos_npts) for i in range(dos_npts)]
    sh = obs.get("spectrum_history")
    specs = [[sh[i][m] for i in range(volume)] for m in range(nmeas)] if sh else None
    if measure_history and sh:   # prog/data_save.hxx:266-345
        def dos0(spec, z):
            d = 0j
            for ev in spec:
                d += 1. / (complex(z, 0.) - ev + complex(0., dos_offset))
            return -(d.imag / volume) / math.pi
        data = [dos0(s, 0.0) for s in specs]
        rows = accumulate_binning(data[::-1], mb)
        save_binning(rows, "dos0")
        db = estimate_bin(rows)
        tab = []
        for z in grid:
            data = [dos0(s, z) for s in specs]
            st = calc_stats(binned(data[::-1], db))
            tab.append([z, st[1], st[3]])
        out["tables"]["dos_err"] = tab
        fermi = lambda w: 1.0 / (1.0 + math.exp(beta * w))
        nc = ncerr = 0.0
        for i in range(len(grid) - 1):
            h = grid[i + 1] - grid[i]
            f0, f1 = fermi(grid[i]), fermi(grid[i + 1])
            nc += 0.5 * h * (tab[i][1] * f0 + tab[i + 1][1] * f1)
            ncerr += 0.5 * h * ((tab[i][2] * f0) ** 2 + (tab[i + 1][2] * f1) ** 2)
        out["stats"]["nc"] = (db, (0, nc, 0.0, math.sqrt(ncerr)))
    ih = obs.get("ipr_history")
    if measure_ipr and ih and sh:   # prog/data_save.hxx:486-530
        iprs = [[ih[i][m] for i in range(volume)] for m in range(nmeas)]

        def ipr_f(spec, ipr, z):
            nom = den = 0.0
            for i in range(volume):
                p = ipr[i] * ipr[i]
                state = p * p
                wme = z - spec[i]
                lor = dos_offset / (wme * wme + dos_offset * dos_offset)
                den += lor
                nom += lor * state
            return nom / den
        data = [ipr_f(specs[m], iprs[m], 0.0) for m in range(nmeas)]
        rows = accumulate_binning(data[::-1], mb)
        save_binning(rows, "ipr0")
        b0 = estimate_bin(rows)
        tab = []
        for z in grid:
            data = [ipr_f(specs[m], iprs[m], z) for m in range(nmeas)]
            st = calc_stats(binned(data[::-1], b0))
            tab.append([z, st[1], st[3]])
        out["tables"]["ipr_err"] = tab
    stiff = obs.get("stiffness")
    if measure_stiffness and stiff:   # prog/data_save.hxx:425-484
        save_binning(accumulate_binning(stiff[::-1], mb), "stiffness")
        w = list(wgrid_cond)
        ch = obs.get("cond_history")
        if len(w) >= 3 and ch and len(ch) == len(w):
            cs0 = accumulate_binning(ch[len(w) // 2], mb)
            cb = estimate_bin(cs0)
            wc = []
            for i in range(len(w)):
                st = calc_stats(binned(ch[i], cb))
                wc.append([w[i], st[1], st[3]])
            out["tables"]["wcond_err"] = wc
            iz = (len(w) - 1) // 2
            c0 = (-wc[iz - 1][1] / w[iz - 1] + -wc[iz + 1][1] / w[iz + 1]) / 2
            c0e = wc[iz + 1][2] / w[iz + 1]
            size0 = cs0[cb][0]
            out["stats"]["cond0"] = (cb, (size0, c0, size0 * c0e * c0e, c0e))
            ce = [[r[0], -r[1] / wi, -r[2] / wi] for r, wi in zip(wc, w)]
            out["tables"]["cond_err"] = ce
            out["tables"]["cond_dynamic"] = [[r[0], r[1] - c0, r[2]] for r in ce]
    return out
