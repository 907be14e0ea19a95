"""Database reader and network assembly (CPU)."""
import os

import numpy as np
import pytest

import kat
from pflotran_gb300 import database

REF_DB = "/root/reference/database/hanford.dat"


def _write_small_db(path):
    """A database in PFLOTRAN's format with the calcite system's rows as the
    known-answer fixture records them."""
    fx = kat.load("kat_calcite_kinetics.json")
    temps = fx["temperatures"]
    q = lambda s: f"'{s}'"
    lines = [f"'temperature points' {len(temps)} " + " ".join(str(t) for t in temps)]
    for p in fx["primaries"]:
        lines.append(f"{q(p['name'])} {p['a0']} {p['Z']} 1.0")
    lines.append("'null' 0 0 0")
    for c in fx["complexes"]:
        st = " ".join(f"{v} {q(s)}" for s, v in c["stoich"])
        lines.append(f"{q(c['name'])} {len(c['stoich'])} {st} " + " ".join(str(k) for k in c["logK"]) +
                     f" {c['a0']} {c['Z']} 1.0")
    lines.append("'null' 1 0. '0' " + " ".join("0." for _ in temps))
    lines.append("'null' 0. 1 0. '0' " + " ".join("0." for _ in temps))
    for m in fx["minerals"]:
        st = " ".join(f"{v} {q(s)}" for s, v in m["stoich"])
        lines.append(f"{q(m['name'])} {m['molar_vol_cm3']} {len(m['stoich'])} {st} " +
                     " ".join(str(k) for k in m["logK"]) + " 100.0")
    lines.append("'null' 0. 1 0. '0' " + " ".join("0." for _ in temps))
    lines.append("'null' 1 0. '0' " + " ".join("0." for _ in temps))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return fx


def test_network_from_database_matches_fixture_network(oracle, tmp_path):
    path = tmp_path / "calcite.dat"
    fx = _write_small_db(path)
    db = database.read_database(path)
    prim = [p["name"] for p in fx["primaries"]]
    net = database.network_from_database(
        db, prim, kinetic_minerals={m["name"]: dict(rate_constant=fx["rate_constant"]) for m in fx["minerals"]},
        debye=kat.debye_25C())
    ref = kat.build_network(fx, oracle)
    a, b = net.build(), ref.build()
    for key in ("eqcplxspecid", "eqcplxstoich", "eqcplx_logK", "eqcplx_Z", "kinmnrlspecid", "kinmnrl_logK",
                "kinmnrl_molar_vol"):
        np.testing.assert_array_equal(np.asarray(a[key]), np.asarray(b[key]), err_msg=key)
    # the Maier-Kelly fit against the oracle's restatement of ReactionFitLogKCoef:
    # the normal equations are ill-conditioned, so compare log K(T), not the coefficients
    ca = np.asarray(a["eqcplx_logKcoef"]).reshape(-1, 5)
    cb = np.asarray(b["eqcplx_logKcoef"]).reshape(-1, 5)
    fitted = [i for i, c in enumerate(fx["complexes"]) if sum(abs(k - 500.0) > 1e-10 for k in c["logK"]) >= 5]
    assert fitted
    for t in (10.0, 25.0, 60.0, 100.0):
        np.testing.assert_allclose([oracle.interpolate_logK(ca[i], t) for i in fitted],
                                   [oracle.interpolate_logK(cb[i], t) for i in fitted], rtol=0, atol=1e-7)


def test_fit_logK_skips_missing_temperatures(oracle):
    temps = [0.0, 25.0, 60.0, 100.0, 150.0, 200.0, 250.0, 300.0]
    logK = [14.9, 13.99, 13.0, 12.25, 11.6, 11.3, 11.2, 500.0]
    c = database.fit_logK(temps, logK)
    ref = oracle.fit_logK(temps, logK)
    for t in temps[:-1] + [37.0]:
        assert abs(oracle.interpolate_logK(np.asarray(c), t) - oracle.interpolate_logK(np.asarray(ref), t)) < 1e-7
    assert database.fit_logK(temps, [500.0] * 4 + [1.0] * 4) is None


@pytest.mark.skipif(not os.path.exists(REF_DB), reason="reference database not present")
def test_reads_reference_database():
    db = database.read_database(REF_DB)
    assert len(db.temperatures) == 8 and db.temperatures[1] == 25.0
    assert {"H+", "Ca++", "HCO3-"} <= set(db.primaries)
    assert "CaCO3(aq)" in db.secondary and "Calcite" in db.minerals
    net = database.network_from_database(db, ["H+", "Ca++", "HCO3-"],
                                         kinetic_minerals={"Calcite": dict(rate_constant=1e-9)})
    names = [c.extra["name"] for c in net.complexes]
    assert "OH-" in names and "CO2(aq)" in names and "CaCO3(aq)" in names
    with pytest.raises(ValueError, match="basis swap"):
        database.network_from_database(db, ["H+", "SO4--"], secondary=["HS-"])
