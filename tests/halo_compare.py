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
INT_FIELDS = ["num_p", "num_child_particles", "n_core", "flags", "desc"]
# extra_halo_info links: indices into the halo output, compared through the
# membership matching
LINK_FIELDS = ["child", "next_cochild", "prev_cochild", "sub_of"]


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


def compare(ref_sets, ref_H, got_sets, got_H, tol=1e-4, fields=FLOAT_FIELDS, ref_E=None,
            got_E=None):
    """Returns (n_unmatched_ref, n_unmatched_got, {field: (worst rel err, ref halo)},
    [ (field, ref halo, err) over tolerance ]).  Every integer field is
    compared exactly; with the extra_halo_info arrays, so are the links
    (mapped through the membership matching: a link to a halo without
    particles must point to a halo without particles on the other side), ph,
    and max_metric within the tolerance."""
    common = set(ref_sets) & set(got_sets)
    g2r = {got_sets[k]: ref_sets[k] for k in common}
    worst, bad = {}, []
    for k in common:
        ri, gi = ref_sets[k], got_sets[k]
        a, b = ref_H[ri], got_H[gi]
        for f in fields:
            e = rel_err(a[f], b[f])
            if e > worst.get(f, (0.0, -1))[0]:
                worst[f] = (e, ri)
            if e > tol:
                bad.append((f, ri, e))
        for f in INT_FIELDS:
            if int(a[f]) != int(b[f]):
                bad.append((f, ri, abs(int(a[f]) - int(b[f]))))
        if ref_E is None:
            continue
        ea, eb = ref_E[ri], got_E[gi]
        for f in LINK_FIELDS:
            rv, gv = int(ea[f]), int(eb[f])
            if rv < 0 or gv < 0:
                ok = rv == gv
            elif gv in g2r:
                ok = g2r[gv] == rv
            else:
                ok = ref_H[rv]["num_p"] <= 0 and got_H[gv]["num_p"] <= 0
            if not ok:
                bad.append((f, ri, 1))
        if int(ea["ph"]) != int(eb["ph"]):
            bad.append(("ph", ri, 1))
        e = rel_err(ea["max_metric"], eb["max_metric"])
        if e > tol:
            bad.append(("max_metric", ri, e))
    return len(set(ref_sets) - common), len(set(got_sets) - common), worst, bad


def membership_diff(ref_sets, got_sets):
    """Particles whose halo differs: the members of the halos of either side
    that have no halo with the same members on the other side (the larger
    of the two counts)."""
    ua = set(ref_sets) - set(got_sets)
    ub = set(got_sets) - set(ref_sets)
    na = sum(len(k) // 8 for k in ua)
    nb = sum(len(k) // 8 for k in ub)
    return max(na, nb)
