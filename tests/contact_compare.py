"""Pair-by-pair comparison of contact sets against the reference's
PxGenerateContacts (fresh caches), with the tolerance the GB300 build claims:
for every pair kind (sphere, plane, capsule, box and convex cores in all
combinations, including the GJK/EPA paths of capsule-box, edge-edge box-box
and the convex cores) the same contact count and every value (normal,
separation, point) within 1e-5.  The oracle and the
device code reproduce the reference's evaluation order, including its
approximate reciprocal in box-box edge clipping, so the observed difference is
0; the 1e-5 bound is the claim.
"""
import numpy as np

NAMES = {0: "sphere", 1: "plane", 2: "capsule", 3: "box"}
CORES = ("point", "segment", "box", "ellipsoid", "cylinder", "cone")   # PxConvexCore::Type
CONTACT_TOL = 1e-5


def shape_name(t):
    t = int(t)
    if t & 0xff == 4:   # convex core: PxConvexCore::Type in bits 8..15
        return "convex_" + CORES[t >> 8]
    return NAMES[t]


def kind(t0, t1):
    a, b = sorted((int(t0), int(t1)), key=lambda t: (t & 0xff, t >> 8))
    return shape_name(a) + "-" + shape_name(b)


def unpack(counts, packed):
    out, k = [], 0
    for c in counts:
        out.append(packed[k:k + c])
        k += c
    return out


def compare(pairs, ref_counts, ref_contacts, counts, contacts):
    """ref_contacts/contacts: list of (c, 8) arrays per pair.  Returns a report dict
    per pair kind: pairs, ok, bad, maxdiff."""
    rep = {}
    for i in range(len(ref_counts)):
        k = kind(pairs["type0"][i], pairs["type1"][i])
        r = rep.setdefault(k, dict(pairs=0, ok=0, bad=0, maxdiff=0.0))
        r["pairs"] += 1
        R, O = ref_contacts[i][:, :7], contacts[i][:, :7]
        if len(R) != len(O):
            r["bad"] += 1
            continue
        d = float(np.abs(R - O).max()) if len(R) else 0.0
        r["maxdiff"] = max(r["maxdiff"], d)
        r["ok" if d <= CONTACT_TOL else "bad"] += 1
    return rep


def assert_report(rep):
    for k, r in rep.items():
        assert r["bad"] == 0, (k, r)
