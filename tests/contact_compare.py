"""Pair-by-pair comparison of contact sets against the reference's
PxGenerateContacts (fresh caches), with the tolerances the GB300 build claims:

* sphere-sphere/plane/capsule/box, plane-capsule, plane-box, capsule-capsule:
  same count, every value (normal, separation, point) within 1e-5;
* box-box: the reference clips incident edges with an approximate reciprocal
  (rcpps, relative error <= 1.5 * 2^-12, physx/source/geomutils/src/pcm/
  GuPCMContactBoxBox.cpp:140) while this build divides exactly, so clipped
  points may move by up to 3.7e-4 of the clipped edge: points/separations are
  matched within 1e-5 + 7.4e-4 * (largest half extent); normals within 1e-5.
  That small shift can flip a near-tie in the 4-point manifold reduction, so a
  bounded fraction of box-box pairs (reported) may pick a different point set;
  the reference's GJK/EPA fallback for edge-edge box pairs (a single point) is
  not reproduced yet and those pairs are reported separately;
* capsule-box: not generated yet by the GB300 build (reported, must be empty).
"""
import numpy as np

NAMES = {0: "sphere", 1: "plane", 2: "capsule", 3: "box"}


def kind(t0, t1):
    a, b = sorted((int(t0), int(t1)))
    return NAMES[a] + "-" + NAMES[b]


def unpack(counts, packed):
    out, k = [], 0
    for c in counts:
        out.append(packed[k:k + c])
        k += c
    return out


def compare(pairs, ref_counts, ref_contacts, counts, contacts):
    """ref_contacts/contacts: list of (c, 8) arrays per pair.  Returns a report dict."""
    rep = {}
    for i in range(len(ref_counts)):
        k = kind(pairs["type0"][i], pairs["type1"][i])
        r = rep.setdefault(k, dict(pairs=0, ok=0, bad=0, gap=0, maxdiff=0.0))
        r["pairs"] += 1
        R, O = ref_contacts[i][:, :7], contacts[i][:, :7]
        if k == "capsule-box":
            r["gap"] += 1
            if len(O) == 0:
                r["ok"] += 1
            else:
                r["bad"] += 1
            continue
        if k == "box-box":
            if len(R) != len(O):
                if len(R) == 1 and len(O) == 0:
                    r["gap"] += 1
                else:
                    r["bad"] += 1
                continue
            he = max(float(np.max(pairs["geom0"][i][:3])), float(np.max(pairs["geom1"][i][:3])))
            tol = 1e-5 + 7.4e-4 * he
            good = True
            for c in R:
                d = np.abs(O - c)
                m = (d[:, :3].max(axis=1) <= 1e-5) & (d[:, 3:7].max(axis=1) <= tol)
                if not m.any():
                    good = False
                    break
            r["ok" if good else "bad"] += 1
            if good and len(R):
                r["maxdiff"] = max(r["maxdiff"], float(min(np.abs(O - c).max() for c in R)))
            continue
        if len(R) != len(O):
            r["bad"] += 1
            continue
        d = float(np.abs(R - O).max()) if len(R) else 0.0
        r["maxdiff"] = max(r["maxdiff"], d)
        r["ok" if d <= 1e-5 else "bad"] += 1
    return rep


def assert_report(rep, box_box_bad_frac=0.03):
    for k, r in rep.items():
        if k == "box-box":
            assert r["bad"] <= box_box_bad_frac * r["pairs"], (k, r)
        elif k == "capsule-box":
            assert r["bad"] == 0, (k, r)
        else:
            assert r["bad"] == 0, (k, r)
