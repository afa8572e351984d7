"""Generate the golden fixtures in this folder by running the REFERENCE implementation itself.

Run from the repository root, in a container where the reference tree is mounted:

    MESHES_REF=/path/to/reference make -C oracle ref
    python tests/golden/make_golden.py [/path/to/reference]     # default: $MESHES_REF

The reference package (``mesh.py`` + ``crossing.py`` + geometry classes) is imported from its own tree
with two stand-ins, because neither library is installed here: ``numba.njit`` as the identity and an empty
``matplotlib.pyplot``.  Its C backend (``mesh.py:82-95``) is pointed at
``oracle/_ref/dot.so``, so every number stored here comes from the reference's own
``StructuredMeshNetwork.dot`` / ``dot_vjp`` (complex128, ``mesh.py:351-392``) and its complex64
``meshdot_helper32`` (``mesh.py:97-113``).  Back-propagation runs with one OpenMP thread
(``mesh.OMP_THREADS = 1``) because the reference's threaded mode-2 reduction races (``c/dot.cpp:135,
281-284``).

Fixtures are small ``.npz`` files; fields are stored (B, N), parameters in the GPU grid layout
(L, N//2, n_p) used by ``gpu/mesh.py:77-81``.
"""
import ctypes
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.meshes_oracle import flat_to_grid, butterfly_strides  # noqa: E402


def import_reference(path):
    nb = types.ModuleType("numba")
    nb.njit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    sys.modules["numba"] = nb
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    spec = importlib.util.spec_from_file_location("meshes", os.path.join(path, "__init__.py"),
                                                  submodule_search_locations=[path])
    m = importlib.util.module_from_spec(spec)
    sys.modules["meshes"] = m
    spec.loader.exec_module(m)
    mm = sys.modules["meshes.mesh"]
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "dot.so"))
    for name in ("meshdot_helper32", "meshdot_helper64"):
        h = getattr(lib, name)
        h.argtypes = (ctypes.c_int,) * 4 + (ctypes.c_void_p,) * 10 + (ctypes.c_int,) * 4
        setattr(mm, name, h)
    mm.BACKEND = "c"
    mm.OMP_THREADS = 1
    return m


def main(ref_path, only=None):
    """Write every fixture, or with only = [group, ...] just those groups of the later case functions
    (converter, configure, direct), leaving the other files untouched."""
    meshes = import_reference(ref_path)
    mm = sys.modules["meshes.mesh"]
    from meshes.clements import ClementsNetwork
    from meshes.reck import ReckNetwork
    from meshes.butterfly import ButterflyNetwork
    from meshes.crossing import MZICrossing, SymCrossing

    rng = np.random.default_rng(20240501)
    written = []

    def save(name, **kw):
        fn = os.path.join(HERE, name + ".npz")
        np.savez_compressed(fn, **kw)
        written.append(fn)

    if only:
        groups = {"converter": converter_cases, "configure": configure_cases, "direct": direct_cases,
                  "errcorr": errcorr_cases}
        for g in only:
            groups[g](save)
        print("wrote", *written, sep="\n  ")
        return

    def nn_case(name, net, N, B, crossing="mzi", diff=True):
        n_p, n_s = {"mzi": (2, 2), "sym": (2, 1)}[crossing]
        lens, shifts = list(map(int, net.lens)), list(map(int, net.shifts))
        n_cr = sum(lens)
        # float32-representable parameters so the GPU grid holds them exactly
        p_cr = rng.uniform(0, 2 * np.pi, (n_cr, n_p)).astype(np.float32).astype(np.float64)
        net.p_phase[:n_cr * n_p] = p_cr.reshape(-1)
        if net.is_phase:
            net.p_phase[n_cr * n_p:] = 0.0
        if net.p_splitter.ndim:
            sp = net.p_splitter.astype(np.float32).astype(np.float64)
            net.p_splitter = sp
        x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        x /= np.linalg.norm(x, axis=1, keepdims=True)
        y = net.dot(x.T).T
        out = dict(N=N, L=len(lens), crossing=crossing, lens=np.array(lens), shifts=np.array(shifts),
                   p=flat_to_grid(p_cr, lens, shifts, N, n_p),
                   x=x, y=y)
        if net.p_splitter.ndim:
            out["s"] = flat_to_grid(net.p_splitter.reshape(n_cr, n_s), lens, shifts, N, n_s)
        if diff:
            dp_cr = rng.standard_normal((n_cr, n_p))
            dp_full = np.zeros(net.n_phase)
            dp_full[:n_cr * n_p] = dp_cr.reshape(-1)
            y2, dy = net.dot(x.T, dp=dp_full)
            out["dp_dir"] = flat_to_grid(dp_cr, lens, shifts, N, n_p)
            out["dy"] = dy.T
            t = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
            g = 2 * (y - t)
            dJdp, dJdv = net.dot_vjp(y.T, g.T)
            out["g"] = g
            out["dJdp"] = flat_to_grid(dJdp[:n_cr * n_p].reshape(n_cr, n_p), lens, shifts, N, n_p)
            out["g_in"] = dJdv.T
            # complex64 arithmetic of the reference C backend (meshdot_helper32) on the same forward
            T = np.ascontiguousarray(net.X.T(p_cr, net.p_splitter if net.p_splitter.ndim else 0.))
            inds = np.array(net.inds, dtype=np.int32)
            v32 = np.ascontiguousarray(x.T.astype(np.complex64))
            ph = np.zeros(N, dtype=np.float32)
            mm.meshdot_helper_c(T.astype(np.complex64), np.empty((0, 0, 0), np.complex64), ph[:0],
                                np.empty((0,), np.float32), v32, np.empty((0, 0), np.complex64), inds,
                                np.array(lens, np.int32), np.array(shifts, np.int32), np.empty((0, 0), np.int32),
                                -1, 0)
            out["y_c64"] = v32.T
        save(name, **out)

    # Clements, MZI with splitter errors
    N = 8
    net = ClementsNetwork(N=N, is_phase=False, phi_out=None, p_splitter=rng.normal(0, 0.02, (N * (N - 1) // 2, 2)))
    nn_case("clements_mzi_N8_split", net, N, 5)
    # Clements, ideal splitters, odd batch
    N = 16
    net = ClementsNetwork(N=N, is_phase=False, phi_out=None)
    nn_case("clements_mzi_N16", net, N, 7)
    # Clements N=64 (the plain-forward shape with a small batch)
    N = 64
    net = ClementsNetwork(N=N, is_phase=False, phi_out=None, p_splitter=rng.normal(0, 0.02, (N * (N - 1) // 2, 2)))
    nn_case("clements_mzi_N64_split", net, N, 16)
    # Reck triangle, splitter errors
    N = 10
    net = ReckNetwork(N=N, p_splitter=rng.normal(0, 0.02, (N * (N - 1) // 2, 2)))
    nn_case("reck_mzi_N10_split", net, N, 6)
    # symmetric crossing (forward only: the reference CPU SymCrossing has no dT)
    N = 8
    net = ClementsNetwork(N=N, is_phase=False, phi_out=None, X=SymCrossing(),
                          p_splitter=rng.normal(0, 0.02, (N * (N - 1) // 2, 1)))
    nn_case("clements_sym_N8_split", net, N, 4, crossing="sym", diff=False)

    # Butterfly (reference form: N-1 layers of adjacent MZIs between permutations)
    N = 16
    bf = ButterflyNetwork(N=N, p_splitter=rng.normal(0, 0.02, (N // 2 * (N - 1), 2)))
    L = N - 1
    n_cr = L * (N // 2)
    p_cr = rng.uniform(0, 2 * np.pi, (n_cr, 2)).astype(np.float32).astype(np.float64)
    bf.p_phase[:n_cr * 2] = p_cr.reshape(-1)
    bf.p_phase[n_cr * 2:] = 0.0
    bf.p_splitter = bf.p_splitter.astype(np.float32).astype(np.float64)
    B = 6
    x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    y = bf.dot(x.T).T
    t = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
    g = 2 * (y - t)
    dJdp, dJdv = bf.dot_vjp(y.T, g.T)
    save("butterfly_mzi_N16_split", N=N, L=L, crossing="mzi", strides=np.array(butterfly_strides(N)),
         p=p_cr.reshape(L, N // 2, 2), s=bf.p_splitter.reshape(L, N // 2, 2), x=x, y=y, g=g,
         dJdp=dJdp[:n_cr * 2].reshape(L, N // 2, 2), g_in=dJdv.T)

    # Lossy generic MZI (crossing.py:444-488: phase errors and gains g_ij < 0) on a Clements mesh: the
    # reference's forward dot only.  Its dot_vjp raises NotImplementedError for this crossing (no dT),
    # so the lossy gradient is pinned by complex128 central differences in the tests instead.
    from meshes.crossing import MZICrossingGeneric
    N = 8
    n_cr = N * (N - 1) // 2
    sp = np.zeros((n_cr, 14))
    sp[:, :2] = rng.normal(0, 0.02, (n_cr, 2))
    sp[:, 2:10] = rng.normal(0, 0.05, (n_cr, 8))
    sp[:, 10:] = -np.abs(rng.normal(0.1, 0.05, (n_cr, 4)))
    sp = sp.astype(np.float32).astype(np.float64)
    net = ClementsNetwork(N=N, is_phase=False, phi_out=None, X=MZICrossingGeneric(), p_splitter=sp)
    lens, shifts = list(map(int, net.lens)), list(map(int, net.shifts))
    p_cr = rng.uniform(0, 2 * np.pi, (n_cr, 2)).astype(np.float32).astype(np.float64)
    net.p_phase[:n_cr * 2] = p_cr.reshape(-1)
    B = 5
    x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    y = net.dot(x.T).T
    T = np.moveaxis(np.asarray(net.X.T(p_cr, sp)), -1, 0)                # (n_cr, 2, 2)
    save("clements_mzigeneric_N8_lossy", N=N, L=len(lens), crossing="mzi_generic", lens=np.array(lens),
         shifts=np.array(shifts), p=flat_to_grid(p_cr, lens, shifts, N, 2), s=flat_to_grid(sp, lens, shifts, N, 14),
         T=flat_to_grid(T.reshape(n_cr, 4), lens, shifts, N, 4).reshape(len(lens), N // 2, 2, 2), x=x, y=y)

    # Phase screen (is_phase=True, phi_pos 'out' and 'in'; c/dot.cpp:97-143): forward, forward-mode
    # derivative and dot_vjp of the reference, screen phases nonzero.
    for pos in ("out", "in"):
        N = 8
        n_cr = N * (N - 1) // 2
        net = ClementsNetwork(N=N, is_phase=True, phi_pos=pos, p_splitter=rng.normal(0, 0.02, (n_cr, 2)))
        lens, shifts = list(map(int, net.lens)), list(map(int, net.shifts))
        net.p_phase[:] = rng.uniform(0, 2 * np.pi, net.p_phase.shape).astype(np.float32).astype(np.float64)
        net.p_splitter = net.p_splitter.astype(np.float32).astype(np.float64)
        B = 5
        x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        x /= np.linalg.norm(x, axis=1, keepdims=True)
        y = net.dot(x.T).T
        dp_full = rng.standard_normal(net.n_phase)
        _, dy = net.dot(x.T, dp=dp_full)
        t = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        g = 2 * (y - t)
        dJdp, dJdv = net.dot_vjp(y.T, g.T)
        save("clements_mzi_N8_screen_" + pos, N=N, L=len(lens), crossing="mzi", phi_pos=pos, lens=np.array(lens),
             shifts=np.array(shifts), p=flat_to_grid(net.p_phase[:n_cr * 2], lens, shifts, N, 2),
             ph=net.p_phase[n_cr * 2:], s=flat_to_grid(net.p_splitter, lens, shifts, N, 2), x=x, y=y,
             dp_dir=flat_to_grid(dp_full[:n_cr * 2], lens, shifts, N, 2), dph_dir=dp_full[n_cr * 2:], dy=dy.T,
             g=g, dJdp=flat_to_grid(dJdp[:n_cr * 2], lens, shifts, N, 2), dJdph=dJdp[n_cr * 2:], g_in=dJdv.T)

    # Clipped meshes (mesh.py:718-802): SquareNetwork and QRNetwork (square.py, qr.py), phase screen on,
    # random crossing phases, screen phases and splitting errors; ClippedNetwork.dot and grad_L2.
    from meshes.square import SquareNetwork
    from meshes.qr import QRNetwork
    for name, cls in (("squarenet", SquareNetwork), ("qrnet", QRNetwork)):
        n = 4
        net = cls(N=n)
        full = net.full
        n_cr = full.n_cr
        full.p_phase[:] = rng.uniform(0, 2 * np.pi, full.p_phase.shape).astype(np.float32).astype(np.float64)
        full.p_splitter = rng.normal(0, 0.02, (n_cr, 2)).astype(np.float32).astype(np.float64)
        net.p_phase, net.p_splitter = full.p_phase, full.p_splitter
        lens, shifts = list(map(int, full.lens)), list(map(int, full.shifts))
        B = 3
        x = (rng.standard_normal((n, B)) + 1j * rng.standard_normal((n, B)))
        y = net.dot(x)
        Z = rng.standard_normal((net.M, n)) + 1j * rng.standard_normal((net.M, n))
        J, dJdp = net.grad_L2(Z)
        save("clipped_%s_N%d" % (name, n), N=full.N, L=full.L, lens=np.array(lens), shifts=np.array(shifts),
             phi_pos=full.phi_pos, p=flat_to_grid(full.p_crossing, lens, shifts, full.N, 2),
             ph=full.phi_out, s=flat_to_grid(full.p_splitter, lens, shifts, full.N, 2),
             idx_in=np.arange(full.N)[net.idx_in], idx_out=np.arange(full.N)[net.idx_out], x=x, y=y, U_target=Z,
             J=J, dJdp=flat_to_grid(dJdp[:n_cr * 2].reshape(n_cr, 2), lens, shifts, full.N, 2),
             dJdph=dJdp[n_cr * 2:])

    # Permutations between layers (mesh.py:238-277; c/dot.cpp:29-40,150-153,289-292): a Clements layout
    # with random permutations before some layers and after the last, without a screen (dot, forward-mode
    # derivative, dot_vjp) and with an input screen (dot, dot_vjp).
    from meshes.mesh import StructuredMeshNetwork
    for name, is_phase, pos in (("perm_mzi_N8_split", False, "out"), ("perm_mzi_N8_screen_in", True, "in")):
        N = 8
        lens, shifts = [int(x) for x in ClementsNetwork(N=N).lens], [int(x) for x in ClementsNetwork(N=N).shifts]
        L = len(lens)
        n_cr = sum(lens)
        perm = [None] * (L + 1)
        for k in (0, 3, 5, L):
            perm[k] = rng.permutation(N)
        net = StructuredMeshNetwork(N, lens, shifts, p_splitter=rng.normal(0, 0.02, (n_cr, 2)), perm=perm,
                                    phi_pos=pos, is_phase=is_phase)
        net.p_phase[:] = rng.uniform(0, 2 * np.pi, net.p_phase.shape).astype(np.float32).astype(np.float64)
        net.p_splitter = net.p_splitter.astype(np.float32).astype(np.float64)
        B = 5
        x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        x /= np.linalg.norm(x, axis=1, keepdims=True)
        y = net.dot(x.T).T
        dp_full = rng.standard_normal(net.n_phase)
        _, dy = net.dot(x.T, dp=dp_full)
        t = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        g = 2 * (y - t)
        dJdp, dJdv = net.dot_vjp(y.T, g.T)
        perm_rows = np.array([np.arange(N) if r is None else r for r in perm])
        save(name, N=N, L=L, crossing="mzi", phi_pos=pos, is_phase=is_phase, lens=np.array(lens),
             shifts=np.array(shifts), perm=perm_rows, p=flat_to_grid(net.p_phase[:n_cr * 2], lens, shifts, N, 2),
             ph=net.p_phase[n_cr * 2:], s=flat_to_grid(net.p_splitter, lens, shifts, N, 2), x=x, y=y,
             dp_dir=flat_to_grid(dp_full[:n_cr * 2], lens, shifts, N, 2), dph_dir=dp_full[n_cr * 2:], dy=dy.T,
             g=g, dJdp=flat_to_grid(dJdp[:n_cr * 2], lens, shifts, N, 2), dJdph=dJdp[n_cr * 2:], g_in=dJdv.T)

    # PILOSS mesh (piloss.py:18-57): a ClippedNetwork over a 2N-mode mesh of full aligned layers with a
    # permutation before every layer and after the last, output phase screen; ClippedNetwork.dot and
    # grad_L2 of the reference with random phases and splitting errors.
    from meshes.piloss import PilossNetwork
    n = 4
    net = PilossNetwork(N=n)
    full = net.full
    n_cr = full.n_cr
    full.p_phase[:] = rng.uniform(0, 2 * np.pi, full.p_phase.shape).astype(np.float32).astype(np.float64)
    full.p_splitter = rng.normal(0, 0.02, (n_cr, 2)).astype(np.float32).astype(np.float64)
    lens, shifts = list(map(int, full.lens)), list(map(int, full.shifts))
    B = 3
    x = (rng.standard_normal((n, B)) + 1j * rng.standard_normal((n, B)))
    y = net.dot(x)
    Z = rng.standard_normal((net.M, n)) + 1j * rng.standard_normal((net.M, n))
    J, dJdp = net.grad_L2(Z)
    perm_rows = np.array([np.arange(full.N) if r is None else r for r in full.perm])
    save("piloss_N%d" % n, N=full.N, L=full.L, lens=np.array(lens), shifts=np.array(shifts), perm=perm_rows,
         phi_pos=full.phi_pos, p=flat_to_grid(full.p_crossing, lens, shifts, full.N, 2), ph=full.phi_out,
         s=flat_to_grid(full.p_splitter, lens, shifts, full.N, 2), idx_in=np.arange(full.N)[net.idx_in],
         idx_out=np.arange(full.N)[net.idx_out], x=x, y=y, U_target=Z, J=J,
         dJdp=flat_to_grid(dJdp[:n_cr * 2].reshape(n_cr, 2), lens, shifts, full.N, 2), dJdph=dJdp[n_cr * 2:])

    # The reference's other crossing parameterisations (crossing.py:292-611): T of each class on random
    # parameters, and a small Clements mesh of each through StructuredMeshNetwork.dot (and dot_vjp where the
    # class has dT).
    from meshes import crossing as cr
    classes = [("mzi_balanced", cr.MZICrossingBalanced, 2, False), ("mzi_outphase", cr.MZICrossingOutPhase, 2, True),
               ("mzi3", cr.MZICrossing3, 3, False), ("mzi3_outphase", cr.MZICrossing3OutPhase, 3, False),
               ("mzi_generic_outphase", cr.MZICrossingGenericOutPhase, 14, False),
               ("cartesian", cr.CartesianCrossing, 2, True), ("bell", cr.MZICrossingBell, 2, True)]

    def draw(name, k, n_s):
        if name == "cartesian":        # inside the unit disks around (+2, 0) and (-2, 0)
            rho, ang = 0.95 * np.sqrt(rng.uniform(0, 1, k)), rng.uniform(0, 2 * np.pi, k)
            side = np.where(rng.uniform(0, 1, k) < 0.5, 2.0, -2.0)
            pp = np.stack([side + rho * np.cos(ang), rho * np.sin(ang)], 1)
        else:
            pp = rng.uniform(0, 2 * np.pi, (k, 2))
        ss = rng.normal(0, 0.05, (k, n_s))
        if n_s == 14:
            ss[:, 10:] = -np.abs(rng.normal(0.1, 0.05, (k, 4)))
        return pp.astype(np.float32).astype(np.float64), ss.astype(np.float32).astype(np.float64)

    out = {}
    for name, cls, n_s, _ in classes:
        pp, ss = draw(name, 7, n_s)
        out[name + "_p"], out[name + "_s"] = pp, ss
        out[name + "_T"] = np.moveaxis(np.asarray(cls().T(pp, ss)), -1, 0)        # (k, 2, 2)
    save("crossings_T", **out)
    for name, cls, n_s, has_dT in classes:
        N = 6
        lens, shifts = [int(x) for x in ClementsNetwork(N=N).lens], [int(x) for x in ClementsNetwork(N=N).shifts]
        n_cr = sum(lens)
        pp, ss = draw(name, n_cr, n_s)
        net = StructuredMeshNetwork(N, lens, shifts, p_splitter=ss, X=cls(), is_phase=False)
        net.p_phase[:] = pp.reshape(-1)
        B = 4
        x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
        x /= np.linalg.norm(x, axis=1, keepdims=True)
        y = net.dot(x.T).T
        extra = {}
        if has_dT:
            t = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N)))
            g = 2 * (y - t)
            dJdp, dJdv = net.dot_vjp(y.T, g.T)
            extra = dict(g=g, dJdp=flat_to_grid(dJdp.reshape(n_cr, 2), lens, shifts, N, 2), g_in=dJdv.T)
        save("xmesh_%s_N%d" % (name, N), N=N, L=len(lens), crossing=name, lens=np.array(lens),
             shifts=np.array(shifts), p=flat_to_grid(pp, lens, shifts, N, 2), s=flat_to_grid(ss, lens, shifts, N, n_s),
             x=x, y=y, **extra)

    converter_cases(save)
    configure_cases(save)
    direct_cases(save)
    errcorr_cases(save)
    print("wrote", *written, sep="\n  ")


def configure_cases(save):
    """The reference's own self-configuration by matrix diagonalisation (configure.py:187-330): a Reck mesh
    programmed with ReckNetwork(M=U, method='diag*') and (method='diag'), and a SquareNet with
    SquareNetwork(M=M, method='diag'), each from a recorded NumPy seed (diag draws its random start from
    np.random).  Stored: the target, splitting errors (reference flat order), the seed, the programmed
    crossing phases and output screen, and the programmed mesh's matrix.  Own seeded stream."""
    from meshes.reck import ReckNetwork
    from meshes.square import SquareNetwork

    rng = np.random.default_rng(20261205)

    def haar(n):
        Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        Q, R = np.linalg.qr(Z)
        return Q * (np.diag(R) / np.abs(np.diag(R)))[None, :]

    for name, n, method, seed in (("reck_diagstar_N8", 8, "diag*", 11), ("reck_diag_N8", 8, "diag", 12)):
        U = haar(n)
        sp = rng.normal(0, 0.02, (n * (n - 1) // 2, 2)).astype(np.float32).astype(np.float64)
        np.random.seed(seed)
        net = ReckNetwork(M=U, p_splitter=sp, method=method)
        save("configure_" + name, N=n, method=method, seed=seed, U=U, p_splitter=sp, lens=np.array(net.lens),
             shifts=np.array(net.shifts), p_crossing=np.array(net.p_crossing), phi_out=np.array(net.phi_out),
             matrix=net.dot(np.eye(n, dtype=complex)))
    n = 3
    M = 0.8 * haar(n)
    seed = 13
    np.random.seed(seed)
    net = SquareNetwork(M=M, method="diag")
    save("configure_square_diag_N3", N=n, method="diag", seed=seed, M=M, lens=np.array(net.full.lens),
         shifts=np.array(net.full.shifts), p_crossing=np.array(net.full.p_crossing),
         phi_out=np.array(net.full.phi_out), matrix=net.dot(np.eye(n, dtype=complex)))


def direct_cases(save):
    """The reference's direct method (configure.py:333-410): Reck meshes programmed with
    ReckNetwork(M=U, p_splitter=sp, method='direct', phi_pos='in') and SquareNets with
    SquareNetwork(M=M, method='direct', phi_pos='in') (the direct method needs no random draws).  Stored: the
    target, splitting errors (reference flat order), geometry, the programmed crossing phases and input screen,
    and the programmed mesh's matrix.  Own seeded stream."""
    from meshes.reck import ReckNetwork
    from meshes.square import SquareNetwork

    rng = np.random.default_rng(20261206)

    def haar(n):
        Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        Q, R = np.linalg.qr(Z)
        return Q * (np.diag(R) / np.abs(np.diag(R)))[None, :]

    for name, n, sig in (("reck_direct_N8", 8, 0.02), ("reck_direct_N5", 5, 0.0), ("reck_direct_N16", 16, 0.03)):
        U = haar(n)
        sp = rng.normal(0, sig, (n * (n - 1) // 2, 2)).astype(np.float32).astype(np.float64)
        net = ReckNetwork(M=U, p_splitter=sp, method="direct", phi_pos="in")
        save("configure_" + name, N=n, method="direct", U=U, p_splitter=sp, lens=np.array(net.lens),
             shifts=np.array(net.shifts), p_crossing=np.array(net.p_crossing), phi_out=np.array(net.phi_out),
             X=type(net.X).__name__, matrix=net.dot(np.eye(n, dtype=complex)))
    for name, shape, eig in (("square_direct_N3", (3, 3), None), ("square_direct_4x2", (4, 2), 0.9)):
        M = 0.8 * haar(max(shape))[:shape[0], :shape[1]]
        net = SquareNetwork(M=M, method="direct", phi_pos="in", eig=eig)
        save("configure_" + name, method="direct", M=M, eig=-1.0 if eig is None else eig, fact=net.fact,
             lens=np.array(net.full.lens), shifts=np.array(net.full.shifts),
             p_crossing=np.array(net.full.p_crossing), phi_out=np.array(net.full.phi_out),
             X=type(net.full.X).__name__, matrix=net.dot(np.eye(shape[1], dtype=complex)))


def errcorr_cases(save):
    """The reference's local error correction (configure.py:412-433, errcorr_local): a Clements mesh with ideal
    splitters and a permuted nearest-neighbour mesh with splitting errors, both with random phases, each corrected
    for random splitting errors.  Stored: geometry, permutation rows, the target's phases, splitters and screen, the new
    splitting errors, the corrected phases and screen, and both matrices.  Own seeded stream."""
    from meshes.clements import ClementsNetwork
    from meshes.configure import errcorr_local
    from meshes.mesh import StructuredMeshNetwork

    rng = np.random.default_rng(20261207)

    def f32(a):
        return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)

    def record(name, net, sp):
        N = net.N
        p0, s0 = np.array(net.p_crossing), np.array(net.p_splitter) * np.ones((net.n_cr, 2))
        phi0 = np.array(net.phi_out)
        U0 = net.dot(np.eye(N, dtype=complex))
        out = errcorr_local(net, sp)
        rows = np.array([np.arange(N) if r is None else np.asarray(r) for r in net.perm])
        save("errcorr_" + name, N=N, lens=np.array(net.lens), shifts=np.array(net.shifts), perm_rows=rows,
             perm_none=np.array([r is None for r in net.perm]), p_crossing0=p0, p_splitter0=s0, phi_out0=phi0,
             p_splitter=sp, p_crossing=np.array(out.p_crossing), phi_out=np.array(out.phi_out), matrix0=U0,
             matrix=out.dot(np.eye(N, dtype=complex)))

    # (random phases: the decomposition ClementsNetwork(M=U) calls np.nan_to_num with a positional copy=0 on
    # scalars, which NumPy 2 refuses; errcorr_local itself passes arrays)
    net = ClementsNetwork(N=8)
    net.p_crossing[:] = f32(rng.uniform(0, 2 * np.pi, net.p_crossing.shape))
    net.phi_out[:] = f32(rng.uniform(0, 2 * np.pi, 8))
    record("clements_N8", net, f32(rng.normal(0, 0.05, (net.n_cr, 2))))
    N, lens, shifts = 8, [4, 3, 4, 3, 4, 3], [0, 1, 0, 1, 0, 1]
    perm = [None, rng.permutation(N), None, rng.permutation(N), None, None, rng.permutation(N)]
    n_cr = sum(lens)
    net = StructuredMeshNetwork(N, lens, shifts, p_crossing=f32(rng.uniform(0, 2 * np.pi, (n_cr, 2))),
                                phi_out=f32(rng.uniform(0, 2 * np.pi, N)), perm=perm,
                                p_splitter=f32(rng.normal(0, 0.02, (n_cr, 2))))
    record("perm_N8", net, f32(rng.normal(0, 0.05, (n_cr, 2))))


def converter_cases(save):
    """Networks as the reference's StructuredMeshNetwork.gpu() converter sees them (mesh.py:568-579): for each
    reference network the attributes that converter reads (N, L, lens, shifts, grid_phase, grid_splitter, the
    crossing class, perm, is_phase, phi_out, phi_pos; a ClippedNetwork's full mesh and ports) and its own dot /
    dot_vjp outputs.  Own seeded stream, so the fixtures above do not change."""
    from meshes.clements import ClementsNetwork
    from meshes.reck import ReckNetwork
    from meshes.butterfly import ButterflyNetwork
    from meshes.mesh import StructuredMeshNetwork
    from meshes.square import SquareNetwork
    from meshes.crossing import MZICrossingOutPhase

    rng = np.random.default_rng(20261204)

    def f32(a):
        return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)

    def randomise(net):
        net.p_phase[:] = f32(rng.uniform(0, 2 * np.pi, net.p_phase.shape))
        if net.p_splitter.ndim:
            net.p_splitter = f32(rng.normal(0, 0.02, net.p_splitter.shape))

    def attrs(net, prefix=""):
        perm_rows = np.array([np.arange(net.N) if r is None else np.asarray(r) for r in net.perm])
        perm_none = np.array([r is None for r in net.perm])
        return {prefix + "N": net.N, prefix + "L": net.L, prefix + "lens": np.array(net.lens),
                prefix + "shifts": np.array(net.shifts), prefix + "grid_phase": net.grid_phase,
                prefix + "grid_splitter": net.grid_splitter, prefix + "X": type(net.X).__name__,
                prefix + "net_class": type(net).__name__, prefix + "perm_rows": perm_rows,
                prefix + "perm_none": perm_none, prefix + "is_phase": bool(net.is_phase),
                prefix + "phi_out": np.asarray(net.phi_out if net.is_phase else np.zeros(0)),
                prefix + "phi_pos": net.phi_pos}

    def case(name, net, B, vjp=True):
        randomise(net)
        N = net.N
        x = rng.standard_normal((N, B)) + 1j * rng.standard_normal((N, B))
        x /= np.linalg.norm(x, axis=0, keepdims=True)
        y = net.dot(x)
        out = dict(attrs(net), x=x, y=y, p_phase=net.p_phase)
        if vjp:
            t = rng.standard_normal((N, B)) + 1j * rng.standard_normal((N, B))
            g = 2 * (y - t)
            dJdp, dJdv = net.dot_vjp(y, g)
            out.update(g=g, dJdp=dJdp, g_in=dJdv)
        save("converter_" + name, **out)

    n = 8
    case("clements_mzi_N8_screen", ClementsNetwork(N=n, p_splitter=np.zeros((n * (n - 1) // 2, 2))), 5)
    n = 6
    case("reck_mzi_N6_screen", ReckNetwork(N=n, p_splitter=np.zeros((n * (n - 1) // 2, 2))), 4)
    n = 8
    case("butterfly_mzi_N8", ButterflyNetwork(N=n, p_splitter=np.zeros((n // 2 * (n - 1), 2))), 4)
    n = 8
    lens, shifts = [int(v) for v in ClementsNetwork(N=n).lens], [int(v) for v in ClementsNetwork(N=n).shifts]
    perm = [None] * (len(lens) + 1)
    for k in (1, 4, len(lens)):
        perm[k] = rng.permutation(n)
    case("perm_mzi_N8", StructuredMeshNetwork(n, lens, shifts, p_splitter=np.zeros((sum(lens), 2)), perm=perm,
                                              is_phase=False), 3)
    n = 6
    case("outphase_N6", StructuredMeshNetwork(n, [int(v) for v in ClementsNetwork(N=n).lens],
                                              [int(v) for v in ClementsNetwork(N=n).shifts],
                                              p_splitter=np.zeros((n * (n - 1) // 2, 2)), X=MZICrossingOutPhase(),
                                              is_phase=False), 3)
    # a clipped network: SquareNetwork (square.py) over its full diamond mesh, ClippedNetwork.dot and grad_L2
    net = SquareNetwork(N=3)
    full = net.full
    randomise(full)
    net.p_phase, net.p_splitter = full.p_phase, full.p_splitter
    x = rng.standard_normal((net.N, 2)) + 1j * rng.standard_normal((net.N, 2))
    y = net.dot(x)
    Z = rng.standard_normal((net.M, net.N)) + 1j * rng.standard_normal((net.M, net.N))
    J, dJdp = net.grad_L2(Z)
    save("converter_squarenet_N3", **attrs(full, "full_"), net_class="SquareNetwork",
         idx_in=np.arange(full.N)[net.idx_in], idx_out=np.arange(full.N)[net.idx_out], x=x, y=y, U_target=Z, J=J,
         dJdp=dJdp, p_phase=full.p_phase)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    if args:
        main(args[0], only)
    elif os.environ.get("MESHES_REF"):
        main(os.environ["MESHES_REF"], only)
    else:
        sys.exit("usage: make_golden.py [--only=converter|configure|direct|errcorr ...] /path/to/reference "
                 "(or set MESHES_REF)")
