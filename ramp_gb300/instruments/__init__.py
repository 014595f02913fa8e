"""Synthetic instrument definition files (the reference's JSON format) for
the benchmark and parity workloads, and generators for their inputs.

* small_chain.json  — flat-spectrum moderator, 30x30 mm slit, vanadium-like
  incoherent cylinder (r 5 mm, h 40 mm), banana detector r 2.5 m with a
  500 x 500 (2theta 5-135 deg, TOF 0-20 ms) histogram.
* let_like.json     — LET-like direct-geometry chopper spectrometer:
  Maxwellian moderator at 40 K, four m=2 supermirror guide segments, five
  disk choppers phased for $Ei$, optional slit ($use_slit$, $slit_w$),
  powder sample with 40 lines, banana detector r 3.5 m with a 720 x 1000
  (2theta -40..140 deg, TOF 0-50 ms) histogram.
* let_like_misis.json — the LET-like chain fed by the tabulated ISIS
  moderator (MISIS) from a seeded synthetic spectrum file in the McStas/MCNP
  tally format ($spec_file$).
* powder_diffractometer.json — curved PG(002) mosaic monochromator at the
  Bragg angle for $Ei$ ($mono_angle$), one-line powder sphere (SPowder1),
  banana detector with a 1D 2theta histogram (-10..150 deg, 0.1 deg).
* tas_like.json — triple-axis-like: PG(002) monochromator for $Ei$, SRescal
  sample focusing onto a PG(002) analyser set for $Ef$, and a counter.
* mesh_imaging.json — near-parallel flat beam through a seeded perturbed
  torus mesh (GMesh + SAttenuate, mu 0.5 /cm) rotated by $angle$, onto a
  1024 x 1024 pixel detector.
All inputs are seeded synthetic stand-ins; nothing is read from elsewhere.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GENERATED = os.path.join(HERE, "_generated")


def path(name):
    return os.path.join(HERE, name)


def write_flat_sqw(fn, sigma_abs=5.08, sigma_inc=5.08, rho=0.0723, nq=201, qmax=15.0,
                   nw=5, wmax=0.05):
    """A McStas Isotropic_Sqw file with S(q, w) flat in q and peaked at w=0
    (a vanadium-like incoherent scatterer).  The header keeps the
    reference loader's field names; its scattering cross-section is read
    from the ``sigma_coh`` field (isotropic.py:200)."""
    q = np.linspace(0.0, qmax, nq)
    w = np.linspace(-wmax, wmax, nw)
    s = np.exp(-0.5 * (w / (wmax / 2.0)) ** 2)
    with open(fn, "w") as f:
        f.write("# Format: Sqw data file for Isotropic_Sqw (synthetic, vanadium-like)\n")
        f.write("# V_rho %.6f\n" % rho)
        f.write("# sigma_abs %.4f\n" % sigma_abs)
        f.write("# sigma_coh %.4f\n" % sigma_inc)
        f.write("# sigma_inc 0.0\n")
        f.write("# q vector\n")
        f.write(" ".join("%.6f" % v for v in q) + "\n")
        f.write("# w vector\n")
        f.write(" ".join("%.6f" % v for v in w) + "\n")
        f.write("# S(q,w) matrix, one row per q\n")
        for _ in q:
            f.write(" ".join("%.6e" % v for v in s) + "\n")
    return fn


def powder_lines(n=40, seed=7):
    """d-spacings uniform in [0.8, 4] AA and |F|^2 log-uniform over three
    decades, numpy seed 7."""
    rng = np.random.default_rng(seed)
    d = np.sort(rng.uniform(0.8, 4.0, n))
    f2 = 10.0 ** rng.uniform(-1.0, 2.0, n)
    return d, f2


def torus_triangles(R=0.020, r=0.008, nu=448, nv=224, noise=0.0002, seed=5):
    """A closed torus mesh (axis along y) with Gaussian vertex noise:
    2*nu*nv triangles (200,704 for the defaults), float32 [n, 9]."""
    rng = np.random.default_rng(seed)
    u = np.arange(nu) * (2 * np.pi / nu)
    v = np.arange(nv) * (2 * np.pi / nv)
    U, V = np.meshgrid(u, v, indexing="ij")
    X = (R + r * np.cos(V)) * np.cos(U)
    Z = (R + r * np.cos(V)) * np.sin(U)
    Y = r * np.sin(V)
    P = np.stack([X, Y, Z], axis=-1) + rng.normal(0.0, noise, (nu, nv, 3))
    i0, j0 = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    i1, j1 = (i0 + 1) % nu, (j0 + 1) % nv
    a, b, c, d = P[i0, j0], P[i1, j0], P[i1, j1], P[i0, j1]
    # counter-clockwise seen from outside: outward normals, as STL expects
    t1 = np.concatenate([a, c, b], axis=-1).reshape(-1, 9)
    t2 = np.concatenate([a, d, c], axis=-1).reshape(-1, 9)
    return np.concatenate([t1, t2]).astype(np.float32)


def write_isis_spectrum(fn, n_e=60, n_t=100, seed=3, time_offset=150.0):
    """A synthetic moderator spectrum in the McStas/MCNP tally text format the
    reference's MISIS reads: per energy bin (edges in MeV, log-spaced from
    1e-11 to 1e-7), a time histogram of ``t value (error)`` lines (t in
    units of 10 ns, log-spaced 1..1e6) and a total line.  Intensities are a
    Maxwellian-like energy shape times a pulse in time with seeded noise;
    the first energy bin is empty."""
    r = np.random.default_rng(seed)
    edges = np.logspace(-11, -7, n_e + 1)
    t = np.logspace(0, 6, n_t)
    E = 0.5 * (edges[:-1] + edges[1:]) * 1e9                   # meV
    shape_e = (E / 3.0) * np.exp(-E / 3.0) + 0.05 * np.exp(-E / 40.0)
    tau = 2e2 + 2e3 / np.sqrt(E + 0.1)                          # pulse width, 10 ns units
    out = ["1tally 5 nps %d" % 200000, "c synthetic spectrum, seed %d" % seed,
           "c TimeOffset %g" % time_offset]
    for k in range(n_e):
        out += [" surface 9999", "segment:  0", "user bin total",
                "energy bin: %.6e to %.6e" % (edges[k], edges[k + 1]), "cosine:   1", " time "]
        pulse = (t / tau[k]) * np.exp(-t / tau[k])
        vals = 1e-8 * shape_e[k] * pulse * (1.0 + 0.1 * r.standard_normal(n_t)).clip(0.0)
        if k == 0:
            vals[:] = 0.0
        for ti, v in zip(t, vals):
            out.append("%.6e %.6e (%.6e) " % (ti, v, 0.1 * v))
        out.append("  total      %.6e (%.6e)" % (vals.sum(), 0.1 * vals.sum()))
    out.append("1end")
    with open(fn, "w") as f:
        f.write("\n".join(out) + "\n")


def ensure_inputs():
    """Write the generated inputs (Sqw file, torus STL, moderator spectrum)
    if missing."""
    from ..geom.mesh import write_stl
    os.makedirs(GENERATED, exist_ok=True)
    sqw = os.path.join(GENERATED, "vanadium_inc.sqw")
    if not os.path.exists(sqw):
        write_flat_sqw(sqw)
    stl = os.path.join(GENERATED, "torus.stl")
    if not os.path.exists(stl):
        write_stl(stl, torus_triangles())
    spec = os.path.join(GENERATED, "isis_spectrum.mcstas")
    if not os.path.exists(spec):
        write_isis_spectrum(spec)
    return {"sqw": sqw, "stl": stl, "spectrum": spec}


def let_like_kwargs(Ei=3.7, use_slit=0, slit_w=0.03):
    return dict(Ei=Ei, use_slit=use_slit, slit_w=slit_w)


def let_like_misis_kwargs(Ei=3.7, use_slit=0, slit_w=0.03):
    return dict(Ei=Ei, use_slit=use_slit, slit_w=slit_w,
                spec_file=repr(ensure_inputs()["spectrum"]))


def powder_diffractometer_kwargs(Ei=14.7, d_mono=3.355):
    """Incident energy (meV) and the monochromator Bragg angle for it
    (rad): sin(theta) = lambda / 2d, lambda = 9.045 / sqrt(Ei) AA."""
    lam = 9.04456 / np.sqrt(Ei)
    return dict(Ei=Ei, mono_angle=float(np.arcsin(lam / (2.0 * d_mono))))


def tas_like_kwargs(Ei=5.0, Ef=5.0, dE=0.2, sample_angle=0.6, d_mono=3.355):
    """Bragg angles of monochromator and analyser for Ei and Ef (rad), the
    sample's scattering angle and its focusing target (the analyser, 1 m
    away in the sample frame)."""
    def bragg(E):
        return float(np.arcsin(9.04456 / np.sqrt(E) / (2.0 * d_mono)))
    return dict(Ei=Ei, Ef=Ef, dE=dE, mono_angle=bragg(Ei), ana_angle=bragg(Ef),
                sample_angle=sample_angle,
                sample_target=[float(np.sin(sample_angle)), 0.0, float(np.cos(sample_angle))])


def small_chain_kwargs():
    # $...$ values are substituted as text and evaluated (mcramp.py:333-338),
    # so a file name is passed as a Python string literal
    return dict(sqw_file=repr(ensure_inputs()["sqw"]))


def mesh_imaging_kwargs(angle=0.0):
    return dict(stl_file=repr(ensure_inputs()["stl"]), angle=angle)
