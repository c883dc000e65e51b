"""The C host program: powspec.conf keywords, command-line options, the ASCII
reader's formatter / expression / selection semantics (CPU, everything before
the GPU is needed) and the output file format against the reference's own
output on the same catalogue (GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


@pytest.fixture(scope="session")
def cli():
    from powspec_gb300 import buildlib
    if not os.path.exists(buildlib.LIB):
        buildlib.build_lib()
    exe = buildlib.build_cli()
    assert exe and os.path.exists(exe)
    return exe


def run(exe, args, cwd):
    return subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=300)


@pytest.fixture
def workdir(tmp_path):
    for f in ("data.txt", "powspec.conf"):
        shutil.copy(os.path.join(GOLDEN, "cli", f), tmp_path / f)
    return tmp_path


def test_help_and_template(cli, tmp_path):
    r = run(cli, ["-h"], tmp_path)
    assert r.returncode == 0
    for key in ("DATA_CATALOG", "GRID_SIZE", "PARTICLE_ASSIGN", "GRID_INTERLACE", "MULTIPOLE",
                "OUTPUT_AUTO", "--box-size", "-G"):
        assert key in r.stdout
    r = run(cli, ["--template"], tmp_path)
    assert r.returncode == 0 and "BIN_SIZE" in r.stdout and "LINE_OF_SIGHT" in r.stdout


def test_survey_without_randoms_is_refused(cli, workdir):
    r = run(cli, ["-c", "powspec.conf", "--sim", "F", "--pole", "0"], workdir)
    assert r.returncode != 0
    assert "RAND_CATALOG" in r.stderr


def test_existing_output_without_overwrite(cli, workdir):
    (workdir / "exists.txt").write_text("x\n")
    r = run(cli, ["-c", "powspec.conf", "-a", "exists.txt", "-w", "0"], workdir)
    assert r.returncode != 0 and "exists" in r.stderr


@pytest.mark.parametrize("args,msg", [
    (["-p", "[$1, $2]"], "DATA_POSITION"),
    (["-p", "[$1, $2, $9]"], "column 9"),
    (["-p", "[$1, $2, sqrt($3]"], "invalid expression"),
    (["--grid-size", "1"], "GRID_SIZE"),
    (["-n", "7"], "PARTICLE_ASSIGN"),
    (["--pole", "[0, 8]"], "MULTIPOLE"),
    (["--line-of-sight", "[1, 1, 0]"], "unit vector"),
    (["-b", "0"], "BIN_SIZE"),
])
def test_configuration_errors(cli, workdir, args, msg):
    r = run(cli, ["-c", "powspec.conf", "-a", "o.txt"] + args, workdir)
    assert r.returncode != 0
    assert msg in r.stderr


def test_reader_formatter_expressions_selection(cli, workdir):
    # 2 header lines skipped, comment and blank lines ignored, a suppressed
    # string column, arithmetic in the positions, weights from a column and a
    # selection on them: 2 of 3 objects kept.
    (workdir / "d.txt").write_text(
        "# header\nsecond header line\n1.0 x 2.0 3.0 0.5\n4 y 5 6 1.5\n# c\n\n7 z 8 9 2.5\n")
    r = run(cli, ["-c", "powspec.conf", "-d", "d.txt", "--data-skip=2", "--data-comment=#",
                  "--data-formatter=%lf %*s %lf %lf %lf", "-p", "[$1*10, ${2}+1, $3]",
                  "--data-wt-comp=$4", "--data-select=$4 < 2", "-a", "o.txt", "-v", "T"], workdir)
    assert "2 objects read from `d.txt'" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("fmt,msg", [("1", "FITS format is not enabled"),
                                     ("3", "invalid `DATA_FORMAT'")])
def test_unsupported_formats(cli, workdir, fmt, msg):
    r = run(cli, ["-c", "powspec.conf", "-a", "o.txt", "-f", fmt], workdir)
    assert r.returncode != 0 and msg in r.stderr


def _npy_catalogue(workdir):
    a = np.loadtxt(workdir / "data.txt")
    # Fortran order: one contiguous array per column; columns permuted so
    # that the expressions differ from the ASCII run's
    np.save(workdir / "data.npy", np.asfortranarray(a[:, [3, 0, 1, 2]]))
    return a.shape[0]


def test_npy_catalogue_is_read(cli, workdir):
    n = _npy_catalogue(workdir)
    r = run(cli, ["-c", "powspec.conf", "-d", "data.npy", "-f", "2", "-p", "[$2, $3, $4]",
                  "--data-wt-comp=$1", "-a", "o.txt", "-v", "T"], workdir)
    assert "%d objects read from `data.npy'" % n in r.stdout, r.stdout + r.stderr
    r = run(cli, ["-c", "powspec.conf", "-d", "data.npy", "-f", "2", "-p", "[$2, $3, $5]",
                  "-a", "o.txt"], workdir)
    assert r.returncode != 0 and "column 5" in r.stderr


@pytest.mark.gpu
def test_npy_catalogue_gives_the_ascii_result(cli, workdir):
    """The same values as .npy and as ASCII: the same output file."""
    _npy_catalogue(workdir)
    r = run(cli, ["-c", "powspec.conf", "-a", "a.txt"], workdir)
    assert r.returncode == 0, r.stdout + r.stderr
    r = run(cli, ["-c", "powspec.conf", "-d", "data.npy", "-f", "2", "-p", "[$2, $3, $4]",
                  "--data-wt-comp=$1", "-a", "b.txt"], workdir)
    assert r.returncode == 0, r.stdout + r.stderr
    a = (workdir / "a.txt").read_text().splitlines()
    b = (workdir / "b.txt").read_text().splitlines()
    assert len(a) == len(b)
    assert [l for l in a if l.startswith("#")] == [l for l in b if l.startswith("#")]
    ra = [l.split() for l in a if not l.startswith("#")]
    rb = [l.split() for l in b if not l.startswith("#")]
    assert [x[:5] for x in ra] == [x[:5] for x in rb]  # k columns and mode counts
    # P_l: the same mesh; FP32 binning sums may add in another order, and
    # the mu^2 moments carry that order's rounding into P_l at ~1e-7
    pa = np.array([[float(v) for v in x[5:]] for x in ra])
    pb = np.array([[float(v) for v in x[5:]] for x in rb])
    shot = float(a[4].split("Shot noise:")[1].split(",")[0])
    assert (np.abs(pa - pb) / (np.abs(pa[:, :1]) + shot)).max() <= 5e-6


@pytest.mark.gpu
def test_cli_output_matches_reference_file(cli, workdir):
    """Same catalogue and powspec.conf as the reference's run: header lines,
    k columns and mode counts identical; P_l within the FP32 tolerance."""
    os.remove(workdir / "powspec.conf")
    shutil.copy(os.path.join(GOLDEN, "cli", "powspec.conf"), workdir / "powspec.conf")
    r = run(cli, ["-c", "powspec.conf", "-a", "gpu_auto.txt"], workdir)
    assert r.returncode == 0, r.stdout + r.stderr
    got = (workdir / "gpu_auto.txt").read_text().splitlines()
    ref = open(os.path.join(GOLDEN, "cli", "ref_auto.txt")).read().splitlines()
    assert len(got) == len(ref)
    head = [i for i, l in enumerate(ref) if l.startswith("#")]
    for i in head:
        assert got[i] == ref[i]
    shot = float(ref[4].split("Shot noise:")[1].split(",")[0])
    g = np.array([[float(x) for x in l.split()] for l in got if not l.startswith("#")])
    f = np.array([[float(x) for x in l.split()] for l in ref if not l.startswith("#")])
    rows = [l for l in got if not l.startswith("#")]
    rrows = [l for l in ref if not l.startswith("#")]
    for a, b in zip(rows, rrows):  # kcen kmin kmax kavg nmod: same text
        assert a.split()[:5] == b.split()[:5]
    scale = np.abs(f[:, 5]) + shot
    assert (np.abs(g[:, 5:] - f[:, 5:]) / scale[:, None]).max() <= 1e-5


@pytest.fixture
def survey_dir(tmp_path):
    for f in ("data.txt", "rand.txt", "powspec.conf", "powspec_box.conf", "data_radecz.txt",
              "rand_radecz.txt", "z_dist.txt", "powspec_cnvt.conf", "powspec_table.conf",
              "powspec_yama.conf", "powspec_cross.conf", "powspec_yama_il.conf",
              "powspec_yama_nz.conf"):
        shutil.copy(os.path.join(GOLDEN, "survey", f), tmp_path / f)
    return tmp_path


@pytest.mark.parametrize("args,msg", [
    (["--pole", "[0, 7]"], "MULTIPOLE"),
    (["--data-convert", "T"], "OMEGA_M"),
    (["--data-convert", "T", "--omega-m", "1.5"], "OMEGA_M"),
    (["--data-convert", "T", "--omega-m", "0.3", "--eos-w", "-0.2"], "DE_EOS_W"),
    (["--data-convert", "T", "--omega-m", "0.3", "--cmvdst-err", "1e-20"], "CMVDST_ERR"),
    (["--rand-pos", "[$1, $2]"], "RAND_POSITION"),
])
def test_survey_configuration_errors(cli, survey_dir, args, msg):
    r = run(cli, ["-c", "powspec.conf", "-a", "o.txt"] + args, survey_dir)
    assert r.returncode != 0 and msg in r.stderr, r.stderr


def test_survey_needs_nz(cli, survey_dir):
    conf = (survey_dir / "powspec.conf").read_text().replace("DATA_NZ", "#").replace("RAND_NZ", "#")
    (survey_dir / "nonz.conf").write_text(conf)
    r = run(cli, ["-c", "nonz.conf", "-a", "o.txt"], survey_dir)
    assert r.returncode != 0 and "DATA_NZ" in r.stderr


def test_survey_catalogues_are_read(cli, survey_dir):
    r = run(cli, ["-c", "powspec.conf", "-a", "o.txt", "-v", "T"], survey_dir)
    out = r.stdout
    assert "2337 objects read from `data.txt'" in out and "7011 objects read from `rand.txt'" in out
    assert "Box size: [410, 410, 410]" in out, out


def _compare(got_path, ref_path):
    """Header lines, k columns and counts equal; |dP_l| / (|P_0| + shot) per
    row and multipole (shot 0 for cross spectra)."""
    got = open(got_path).read().splitlines()
    ref = open(ref_path).read().splitlines()
    assert len(got) == len(ref)
    assert [l for l in got if l.startswith("#")] == [l for l in ref if l.startswith("#")]
    rows = [l.split() for l in got if not l.startswith("#")]
    rrows = [l.split() for l in ref if not l.startswith("#")]
    assert [x[:5] for x in rows] == [x[:5] for x in rrows]  # k columns and mode counts
    shot = [float(l.split("Shot noise:")[1].split(",")[0]) for l in ref if "Shot noise:" in l]
    g = np.array([[float(v) for v in x[5:]] for x in rows])
    f = np.array([[float(v) for v in x[5:]] for x in rrows])
    return np.abs(g - f) / (np.abs(f[:, :1]) + (shot[0] if shot else 0.0))


def test_converted_survey_catalogues_are_read(cli, survey_dir):
    r = run(cli, ["-c", "powspec_cnvt.conf", "-a", "o.txt", "-v", "T"], survey_dir)
    assert "Legendre-Gauss order" in r.stdout, r.stdout + r.stderr
    assert "Box size: [410, 410, 410]" in r.stdout
    r = run(cli, ["-c", "powspec_table.conf", "-a", "o.txt", "-v", "T"], survey_dir)
    assert "400 comoving distance samples read" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("conf,ref,out", [
    ("powspec.conf", "ref_auto.txt", "-a"), ("powspec_box.conf", "ref_auto_box.txt", "-a"),
    ("powspec_cnvt.conf", "ref_auto_cnvt.txt", "-a"),
    ("powspec_table.conf", "ref_auto_table.txt", "-a"),
    ("powspec_yama.conf", "ref_auto_yama.txt", "-a"),
    ("powspec_cross.conf", "ref_cross_yama.txt", "-x"),
    ("powspec_yama_il.conf", "ref_auto_yama_il.txt", "-a"),
    ("powspec_yama_nz.conf", "ref_auto_yama_nz.txt", "-a")])
def test_survey_matches_reference_file(cli, survey_dir, conf, ref, out):
    """Data minus alpha x randoms with FKP weights in the fitted (or given,
    non-cubic) box, from Cartesian or converted (RA, Dec, z) coordinates;
    multipoles 0, 2, 4 (non-interlaced) auto and cross, and 0 to 6 on the
    interlaced mesh (the c2r of the combined field), and with randoms at
    1.5 x the data's n(z) (the k = 0 mode far from 0): the reference's
    header lines, k columns and mode counts, and P_l within 1e-5 of
    |P_0| + shot noise (bin 0 holds the k = 0 mode)."""
    r = run(cli, ["-c", conf, out, "gpu_out.txt"], survey_dir)
    assert r.returncode == 0, r.stdout + r.stderr
    d = _compare(survey_dir / "gpu_out.txt", os.path.join(GOLDEN, "survey", ref))
    assert d.max() <= 1e-5, d
