"""Halo catalogue comparison used by the parity tests: halos are matched by
their particle membership (the set of particle ids of each halo), then the
fields of matched halos are compared with a relative tolerance."""
import numpy as np

# fields compared for matched halos (float fields with relative tolerance)
FLOAT_FIELDS = ["pos", "corevel", "bulkvel", "m", "r", "child_r", "vmax_r", "mgrav", "vmax",
                "rvmax", "rs", "klypin_rs", "vrms", "J", "energy", "spin", "alt_m", "Xoff",
                "Voff", "b_to_a", "c_to_a", "A", "b_to_a2", "c_to_a2", "bullock_spin",
                "kin_to_pot", "m_pe_b", "m_pe_d", "halfmass_radius", "min_pos_err",
                "min_vel_err", "min_bulkvel_err", "inertia_tensor", "inertia_tensor2", "chi2"]
INT_FIELDS = ["num_p", "num_child_particles", "n_core", "flags"]


def halo_sets(parts, H):
    d = {}
    for i, h in enumerate(H):
        if h["num_p"] <= 0:
            continue
        ids = np.sort(parts["id"][h["p_start"]:h["p_start"] + h["num_p"]])
        d[ids.tobytes()] = i
    return d


def halo_of(parts, H, n):
    lab = np.full(n, -1, np.int64)
    for i, h in enumerate(H):
        if h["num_p"] > 0:
            lab[parts["id"][h["p_start"]:h["p_start"] + h["num_p"]]] = i
    return lab


def sets_from_labels(lab):
    d = {}
    order = np.argsort(lab, kind="stable")
    ls = lab[order]
    cuts = np.flatnonzero(np.diff(ls)) + 1
    for chunk in np.split(order, cuts):
        if len(chunk) and lab[chunk[0]] >= 0:
            d[np.sort(chunk).astype(np.int64).tobytes()] = int(lab[chunk[0]])
    return d


def rel_err(x, y):
    x = np.asarray(x, np.float64).ravel()
    y = np.asarray(y, np.float64).ravel()
    both_nan = np.isnan(x) & np.isnan(y)
    same = (x == y) | both_nan
    den = np.maximum(np.abs(x), np.abs(y))
    den = np.where(den > 0, den, 1.0)
    e = np.where(same, 0.0, np.abs(x - y) / den)
    return float(e.max()) if len(e) else 0.0


def compare(ref_sets, ref_H, got_sets, got_H, tol=1e-4, fields=FLOAT_FIELDS):
    """Returns (n_unmatched_ref, n_unmatched_got, {field: (worst rel err, ref halo)},
    [ (field, ref halo, err) over tolerance ])."""
    common = set(ref_sets) & set(got_sets)
    worst, bad = {}, []
    for k in common:
        a, b = ref_H[ref_sets[k]], got_H[got_sets[k]]
        for f in fields:
            e = rel_err(a[f], b[f])
            if e > worst.get(f, (0.0, -1))[0]:
                worst[f] = (e, ref_sets[k])
            if e > tol:
                bad.append((f, ref_sets[k], e))
        for f in INT_FIELDS:
            if f in fields or f in ("num_p",):
                if int(a[f]) != int(b[f]):
                    bad.append((f, ref_sets[k], abs(int(a[f]) - int(b[f]))))
    return len(set(ref_sets) - common), len(set(got_sets) - common), worst, bad
