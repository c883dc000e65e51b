"""Generate the golden fixtures of tests/golden/ from the REFERENCE itself.

Runs the unmodified reference sources (compiled from source into
oracle/_ref by ``make -C oracle ref``, linked against the FFTW-API shim)
with one OpenMP thread so that every output is deterministic, and stores
inputs + outputs as .npz files.  The reference publishes no test vectors, so
these are the pins of the oracle and of the GPU path:

* ``ref_cases.npz``: seeded catalogues (float64 x, y, z, w) and the
  reference outputs k, kedge, km, cnt, lcnt, pl, xpl, shot, norm for a grid
  of settings (every scheme, interlacing on/off, linear and log bins, all
  poles, auto + cross, KMAX set, tilted line of sight, non-cubic box).
* ``ref_meshes.npz``: the reference density meshes Fr / Frl at Ng = 16 for
  every scheme, interlaced.
* ``cli/``: an ASCII catalogue, a powspec.conf and the reference POWSPEC
  output file for it (the output-format pin).
* ``survey/``: a survey-like data catalogue (a clustered sphere) and its
  randoms, with completeness weights, n(z) and FKP weights, and the
  reference POWSPEC monopole for CUBIC_SIM = F with the box fitted to the
  catalogues (ref_auto.txt) and with BOX_SIZE given (ref_auto_box.txt);
  the same objects as (RA, Dec, z) converted by quadrature
  (ref_auto_cnvt.txt) and by a distance table (ref_auto_table.txt); the
  multipoles 0, 2, 4 on a non-interlaced mesh (ref_auto_yama.txt) and their
  cross spectrum of the catalogue with itself (ref_cross_yama.txt); the
  multipoles 0 to 6 on the interlaced mesh (ref_auto_yama_il.txt); and
  multipoles 0, 2, 4 with randoms at 1.5 x the data's n(z), whose k = 0
  mode is far from 0 (ref_auto_yama_nz.txt); the cross spectrum of the
  catalogue with a 60% subsample of it and half the randoms
  (ref_cross2_il.txt); and log-scale bins (ref_auto_log.txt).

Usage (in a tree that has the reference sources):
    python tests/golden/make_golden.py          # everything
    python tests/golden/make_golden.py survey   # the survey fixture only
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from powspec_gb300 import catalog  # noqa: E402

CASES = [
    # name, ng, assign, interlace, poles, dk, log, kmin, kmax, ncat, box, los, npart, kind
    ("ngp_lin", 16, 0, 0, (0, 2, 4), 0.01, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 3000, "lognormal"),
    ("cic_lin", 16, 1, 0, (0, 2, 4), 0.01, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 3000, "lognormal"),
    ("tsc_il", 16, 2, 1, (0, 2, 4), 0.01, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 3000, "lognormal"),
    ("pcs_il", 16, 3, 1, (0, 2, 4), 0.01, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 3000, "lognormal"),
    ("cic_il_allpoles", 24, 1, 1, (0, 1, 2, 3, 4, 5, 6), 0.008, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 4000, "lognormal"),
    ("tsc_cross", 32, 2, 0, (0, 2, 4), 0.01, 0, 0.0, -1, 2, 1000.0, (0, 0, 1), 5000, "lognormal"),
    ("pcs_il_cross", 32, 3, 1, (0, 2, 4), 0.01, 0, 0.0, -1, 2, 1000.0, (0, 0, 1), 5000, "lognormal"),
    ("cic_log", 32, 1, 1, (0, 2), 0.1, 1, np.log10(0.008), -1, 1, 1000.0, (0, 0, 1), 4000, "lognormal"),
    ("tsc_kmax_los", 32, 2, 1, (0, 2, 4), 0.006, 0, 0.01, 0.07, 1, 1000.0, (0.6, 0, 0.8), 4000, "lognormal"),
    ("cic_kf_edges", 32, 1, 0, (0, 2, 4), 2 * np.pi / 1000.0, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 4000, "uniform"),
    ("cic_noncubic", 16, 1, 0, (0, 2), 0.01, 0, 0.0, -1, 1, (1000.0, 800.0, 1200.0), (0, 0, 1), 3000, "uniform"),
    ("pcs_weights", 32, 3, 1, (0, 2, 4), 0.01, 0, 0.0, -1, 1, 1000.0, (0, 0, 1), 4000, "weighted"),
]


def make_cat(kind, n, box, seed):
    b = np.array(box if isinstance(box, tuple) else (box,) * 3)
    if kind == "uniform":
        c = catalog.uniform(n, box=1.0, seed=seed)
        c[:, :3] = np.minimum(c[:, :3] * b, np.nextafter(b, 0))
        return c
    if kind == "weighted":
        c = catalog.lognormal(n, box=float(b[0]), seed=seed, ngen=32, weights=(0.5, 1.5))
        return c
    return catalog.lognormal(n, box=float(b[0]), seed=seed, ngen=32)


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference sources not found: cannot generate fixtures")
    oracle.build_port()
    oracle.set_threads(1)
    out = {}
    for ci, (name, ng, a, il, poles, dk, lg, kmin, kmax, ncat, box, los, npart, kind) in enumerate(CASES):
        cats = [make_cat(kind, npart, box, 100 + 10 * ci + j) for j in range(ncat)]
        spec = oracle.Spec(ng=ng, box=box, assign=a, interlace=bool(il), poles=poles, los=los,
                           kmin=kmin, kmax=kmax, dk=dk, logscale=bool(lg),
                           isauto=(True, True), iscross=ncat == 2)
        r = oracle.run("ref", spec, cats)
        pre = f"{name}/"
        for j, c in enumerate(cats):
            out[pre + f"cat{j}"] = c
        out[pre + "settings"] = np.array([ng, a, il, dk, lg, kmin, kmax, ncat], dtype=np.float64)
        out[pre + "box"] = np.array(spec.box3())
        out[pre + "los"] = np.array(los, dtype=np.float64)
        out[pre + "poles"] = np.array(poles, dtype=np.int64)
        for f in ("k", "kedge", "km", "cnt", "lcnt", "pl", "xpl", "shot", "norm"):
            out[pre + f] = getattr(r, f)
        print(f"{name}: nbin={r.nbin} N={[len(c) for c in cats]}")
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **out)

    meshes = {}
    cat = make_cat("lognormal", 2000, 1000.0, 7)
    meshes["cat"] = cat
    for a in range(4):
        m0, m1 = oracle.assign("ref", cat, 16, 1000.0, a, 1)
        meshes[f"fr_{a}"] = m0
        meshes[f"frl_{a}"] = m1
    np.savez_compressed(os.path.join(HERE, "ref_meshes.npz"), **meshes)

    # CLI / output-format pin
    cli = os.path.join(HERE, "cli")
    os.makedirs(cli, exist_ok=True)
    cat = make_cat("lognormal", 1500, 500.0, 11)
    np.savetxt(os.path.join(cli, "data.txt"), cat, fmt="%.8f")
    conf = """DATA_CATALOG    = data.txt
DATA_FORMATTER  = "%lf %lf %lf %lf"
DATA_POSITION   = [$1, $2, $3]
DATA_WT_COMP    = $4
CUBIC_SIM       = T
BOX_SIZE        = 500
GRID_SIZE       = 32
PARTICLE_ASSIGN = 2
GRID_INTERLACE  = T
MULTIPOLE       = [0, 2, 4]
BIN_SIZE        = 0.02
OUTPUT_AUTO     = ref_auto.txt
OVERWRITE       = 1
VERBOSE         = F
"""
    with open(os.path.join(cli, "powspec.conf"), "w") as f:
        f.write(conf)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([oracle.REF_CLI, "-c", "powspec.conf"], cwd=cli, check=True, env=env,
                   stdout=subprocess.DEVNULL)
    print("cli fixture written")


SURVEY_CONF = """DATA_CATALOG    = data.txt
RAND_CATALOG    = rand.txt
DATA_FORMATTER  = "%lf %lf %lf %lf %lf"
RAND_FORMATTER  = "%lf %lf %lf %lf %lf"
DATA_POSITION   = [$1, $2, $3]
RAND_POSITION   = [$1, $2, $3]
DATA_WT_COMP    = $4
RAND_WT_COMP    = $4
DATA_WT_FKP     = 1/(1+$5*2000)
RAND_WT_FKP     = 1/(1+$5*2000)
DATA_NZ         = $5
RAND_NZ         = $5
CUBIC_SIM       = F
GRID_SIZE       = 32
PARTICLE_ASSIGN = 3
GRID_INTERLACE  = T
MULTIPOLE       = 0
BIN_SIZE        = 0.02
OUTPUT_AUTO     = {out}
OVERWRITE       = 1
VERBOSE         = F
"""


def survey():
    """Survey fixture: clustered data in a sphere of radius 200 around
    (600, 300, 450), randoms uniform in the sphere (3x), completeness
    weights in [0.8, 1.2], a constant n(z) column and FKP weights
    1 / (1 + n P0), P0 = 2000."""
    if oracle.build_ref() is None:
        raise SystemExit("reference sources not found: cannot generate fixtures")
    d = os.path.join(HERE, "survey")
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(77)
    cen, rad = np.array([600.0, 300.0, 450.0]), 200.0
    c = make_cat("lognormal", 9000, 500.0, 31)[:, :3] - 250.0
    data = c[np.sum(c * c, axis=1) < rad * rad] + cen
    u = rng.uniform(-rad, rad, (12 * len(data), 3))
    rand = u[np.sum(u * u, axis=1) < rad * rad][:3 * len(data)] + cen
    nbar = len(data) / (4.0 / 3.0 * np.pi * rad ** 3)
    for name, pts in (("data.txt", data), ("rand.txt", rand)):
        cols = np.column_stack([pts, rng.uniform(0.8, 1.2, len(pts)), np.full(len(pts), nbar)])
        np.savetxt(os.path.join(d, name), cols, fmt="%.6f %.6f %.6f %.4f %.8e")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    for conf, extra in (("powspec.conf", ""), ("powspec_box.conf", "BOX_SIZE        = [450, 420, 430]\n")):
        out = "ref_auto.txt" if not extra else "ref_auto_box.txt"
        with open(os.path.join(d, conf), "w") as f:
            f.write(SURVEY_CONF.format(out=out) + extra)
        subprocess.run([oracle.REF_CLI, "-c", conf], cwd=d, check=True, env=env,
                       stdout=subprocess.DEVNULL)
    print("survey fixture written:", len(data), "data,", len(rand), "randoms")
    # multipoles l > 0 (non-interlaced mesh): auto, and the cross spectrum
    # of the catalogue with itself
    yama = SURVEY_CONF.replace("GRID_INTERLACE  = T", "GRID_INTERLACE  = F").replace(
        "MULTIPOLE       = 0", "MULTIPOLE       = [0, 2, 4]")
    with open(os.path.join(d, "powspec_yama.conf"), "w") as f:
        f.write(yama.format(out="ref_auto_yama.txt"))
    twice = {"DATA_CATALOG": "[data.txt, data.txt]", "RAND_CATALOG": "[rand.txt, rand.txt]",
             "DATA_FORMATTER": '["%lf %lf %lf %lf %lf", "%lf %lf %lf %lf %lf"]',
             "RAND_FORMATTER": '["%lf %lf %lf %lf %lf", "%lf %lf %lf %lf %lf"]',
             "DATA_POSITION": "[$1, $2, $3, $1, $2, $3]", "RAND_POSITION": "[$1, $2, $3, $1, $2, $3]",
             "DATA_WT_COMP": "[$4, $4]", "RAND_WT_COMP": "[$4, $4]",
             "DATA_WT_FKP": "[1/(1+$5*2000), 1/(1+$5*2000)]",
             "RAND_WT_FKP": "[1/(1+$5*2000), 1/(1+$5*2000)]",
             "DATA_NZ": "[$5, $5]", "RAND_NZ": "[$5, $5]"}
    lines = []
    for line in yama.format(out="").splitlines():
        key = line.split("=")[0].strip()
        if key in twice:
            line = "%-16s= %s" % (key, twice[key])
        elif key == "OUTPUT_AUTO":
            line = "OUTPUT_CROSS    = ref_cross_yama.txt"
        lines.append(line)
    with open(os.path.join(d, "powspec_cross.conf"), "w") as f:
        f.write("\n".join(lines) + "\n")
    # every multipole up to 6 on the interlaced mesh: the harmonics weight the
    # c2r of the combined field
    il = SURVEY_CONF.replace("MULTIPOLE       = 0", "MULTIPOLE       = [0, 1, 2, 3, 4, 5, 6]")
    with open(os.path.join(d, "powspec_yama_il.conf"), "w") as f:
        f.write(il.format(out="ref_auto_yama_il.txt"))
    # randoms with 1.5 x the data's n(z) (and FKP weights from it): the
    # weighted field's total W = F(k = 0) is far from 0, so the k = 0 mode
    # of every multipole counts
    nz = il.replace("RAND_WT_FKP     = 1/(1+$5*2000)", "RAND_WT_FKP     = 1/(1+$5*3000)").replace(
        "RAND_NZ         = $5", "RAND_NZ         = $5*1.5").replace(
        "MULTIPOLE       = [0, 1, 2, 3, 4, 5, 6]", "MULTIPOLE       = [0, 2, 4]")
    with open(os.path.join(d, "powspec_yama_nz.conf"), "w") as f:
        f.write(nz.format(out="ref_auto_yama_nz.txt"))
    # two different catalogues: a 60% subsample of the data with every
    # second random, crossed with the full ones (interlaced, l = 0, 2, 4)
    fmt = "%.6f %.6f %.6f %.4f %.8e"
    dd = np.loadtxt(os.path.join(d, "data.txt"))
    rr = np.loadtxt(os.path.join(d, "rand.txt"))
    np.savetxt(os.path.join(d, "data2.txt"), dd[np.random.default_rng(91).random(len(dd)) < 0.6],
               fmt=fmt)
    np.savetxt(os.path.join(d, "rand2.txt"), rr[::2], fmt=fmt)
    il024 = il.replace("MULTIPOLE       = [0, 1, 2, 3, 4, 5, 6]", "MULTIPOLE       = [0, 2, 4]")
    lines = []
    for line in il024.format(out="").splitlines():
        key = line.split("=")[0].strip()
        if key in twice:
            line = "%-16s= %s" % (key, twice[key])
            line = line.replace("[data.txt, data.txt]", "[data.txt, data2.txt]").replace(
                "[rand.txt, rand.txt]", "[rand.txt, rand2.txt]")
        elif key == "OUTPUT_AUTO":
            line = "OUTPUT_CROSS    = ref_cross2_il.txt"
        lines.append(line)
    with open(os.path.join(d, "powspec_cross2.conf"), "w") as f:
        f.write("\n".join(lines) + "\n")
    # log-scale bins (KMIN 0.01, 0.1 dex), interlaced, l = 0, 2, 4
    lg = il024.replace("BIN_SIZE        = 0.02",
                       "BIN_SIZE        = 0.1\nLOG_SCALE       = T\nKMIN            = 0.01")
    with open(os.path.join(d, "powspec_log.conf"), "w") as f:
        f.write(lg.format(out="ref_auto_log.txt"))
    for conf in ("powspec_yama.conf", "powspec_cross.conf", "powspec_yama_il.conf",
                 "powspec_yama_nz.conf", "powspec_cross2.conf", "powspec_log.conf"):
        subprocess.run([oracle.REF_CLI, "-c", conf], cwd=d, check=True, env=env,
                       stdout=subprocess.DEVNULL)
    survey_converted(d, data, rand, rng, env)


def survey_converted(d, data, rand, rng, env):
    """The same objects as (RA, Dec, redshift) for OMEGA_M = 0.31 (flat,
    w = -1): redshifts from the comoving distance by inverting a fine table
    of the adaptive-quadrature distance.  Run with DATA_CONVERT /
    RAND_CONVERT (Gauss-Legendre, ref_auto_cnvt.txt) and with a
    Z_CMVDST_CNVT table of 400 samples (ref_auto_table.txt)."""
    from scipy import integrate
    om = 0.31

    def dist(z):
        return integrate.quad(lambda t: 2997.92458 / np.sqrt(om * (1 + t) ** 3 + 1 - om), 0, z,
                              epsabs=0, epsrel=1e-13)[0]

    zg = np.linspace(0.0, 0.6, 6001)
    dg = np.array([dist(z) for z in zg])
    for name, pts in (("data_radecz.txt", data), ("rand_radecz.txt", rand)):
        r = np.sqrt(np.sum(pts * pts, axis=1))
        ra = np.degrees(np.arctan2(pts[:, 1], pts[:, 0])) % 360.0
        dec = np.degrees(np.arcsin(pts[:, 2] / r))
        z = np.interp(r, dg, zg)
        cols = np.column_stack([ra, dec, z, rng.uniform(0.8, 1.2, len(pts)),
                                np.full(len(pts), 1e-4)])
        np.savetxt(os.path.join(d, name), cols, fmt="%.9f %.9f %.10f %.4f %.8e")
    zt = np.linspace(0.0, 0.6, 400)
    np.savetxt(os.path.join(d, "z_dist.txt"), np.column_stack([zt, [dist(z) for z in zt]]),
               fmt="%.10f %.10f")
    base = (SURVEY_CONF.replace("data.txt", "data_radecz.txt").replace("rand.txt", "rand_radecz.txt")
            + "DATA_CONVERT    = T\nRAND_CONVERT    = T\n")
    for conf, extra, out in (("powspec_cnvt.conf", "OMEGA_M         = 0.31\n", "ref_auto_cnvt.txt"),
                             ("powspec_table.conf", "Z_CMVDST_CNVT   = z_dist.txt\n", "ref_auto_table.txt")):
        with open(os.path.join(d, conf), "w") as f:
            f.write(base.format(out=out) + extra)
        subprocess.run([oracle.REF_CLI, "-c", conf], cwd=d, check=True, env=env,
                       stdout=subprocess.DEVNULL)
    print("converted survey fixture written")


if __name__ == "__main__":
    if sys.argv[1:] == ["survey"]:
        survey()
    else:
        main()
        survey()
