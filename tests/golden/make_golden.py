"""Generate the golden fixtures in this folder by running PARLA 0.1.4 itself.

Run in a container that holds the reference source tree::

    python tests/golden/make_golden.py <reference source tree> [fixture names ...]

The reference targets NumPy 1.x; two names it uses were removed in NumPy 2
(``np.NaN`` and ``np.row_stack``), so they are restored as aliases before the
import.  Nothing is written into the reference tree (bytecode is disabled).

Each fixture stores the seeded inputs together with the reference outputs, so
the tests that read them never need the reference itself.  Library versions
are recorded because NumPy Generator streams and LAPACK results can change
between releases.
"""
import os
import sys
import warnings

import numpy as np
import scipy

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(path):
    sys.dont_write_bytecode = True
    np.NaN = np.nan
    np.row_stack = np.vstack
    sys.path.insert(0, path)
    import parla  # noqa: F401
    return parla


def _ls_problem(m, n, log_cond, noise, seed):
    """A = U diag(s) V' with logspaced s, b = A x* + noise * unit r_perp."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((m, n))
    U, _ = np.linalg.qr(g)
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.logspace(0, -log_cond, n)
    A = (U * s) @ V.T
    x = rng.standard_normal(n)
    r = rng.standard_normal(m)
    r -= U @ (U.T @ r)
    r /= np.linalg.norm(r)
    b = A @ x + noise * r
    return A, b


def sketches(parla):
    import parla.utils.sketching as usk
    out = {}
    out['ga_wide'] = usk.gaussian_operator(12, 50, np.random.default_rng(11))
    out['ga_tall'] = usk.gaussian_operator(50, 7, np.random.default_rng(12))
    out['ga_raw'] = usk.gaussian_operator(6, 9, np.random.default_rng(10),
                                          normalize=False)
    out['sj_wide'] = usk.sjlt_operator(16, 64, np.random.default_rng(13), 8).toarray()
    out['sj_tall'] = usk.sjlt_operator(64, 16, np.random.default_rng(14), 8).toarray()
    out['sj_nnz3'] = usk.sjlt_operator(20, 300, np.random.default_rng(21), 3).toarray()
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        out['sj_repl'] = usk.sjlt_operator(5, 30, np.random.default_rng(15), 8).toarray()
    rng = np.random.default_rng(16)
    r, e, perm = usk.generate_srct(16, 100, rng)
    out['srct_r'], out['srct_e'], out['srct_perm'] = r, e, perm
    mat = np.random.default_rng(17).standard_normal((100, 5))
    out['srct_in'] = mat
    out['srct_fwd'] = usk.apply_srct(r, e, mat, perm)
    small = np.random.default_rng(18).standard_normal((16, 5))
    out['srct_adj_in'] = small
    out['srct_adj'] = usk.apply_srct(r, e, small, perm, forward=False)
    out['srct_vec'] = usk.apply_srct(r, e, mat[:, 0], perm)
    op = usk.srct_operator(24, 120, np.random.default_rng(22))
    m2 = np.random.default_rng(23).standard_normal((120, 3))
    out['srct_op_in'] = m2
    out['srct_op_out'] = op @ m2
    out['on_tall'] = usk.orthonormal_operator(40, 10, np.random.default_rng(19))
    out['on_wide'] = usk.orthonormal_operator(10, 40, np.random.default_rng(20))
    return out


def lsqr_case(parla):
    from parla.comps.determiter.lsqr import lsqr
    from scipy.sparse.linalg import aslinearoperator
    A, b = _ls_problem(60, 8, 3, 1e-2, 31)
    out = {'A': A, 'b': b}
    for tag, kw in (('plain', dict(atol=1e-12, btol=1e-12, iter_lim=50)),
                    ('lim3', dict(atol=1e-12, btol=1e-12, iter_lim=3)),
                    ('damp', dict(damp=0.3, atol=1e-10, btol=1e-10, iter_lim=50)),
                    ('x0', dict(atol=1e-12, btol=1e-12, iter_lim=50,
                                x0=np.ones(8)))):
        res = lsqr(aslinearoperator(A), b, **kw)
        out[f'{tag}_x'] = res[0]
        out[f'{tag}_istop'] = np.array(res[1])
        out[f'{tag}_itn'] = np.array(res[2])
        out[f'{tag}_arnorms'] = np.asarray(res[7])
    return out


def spo_cases(parla):
    import parla.comps.sketchers.oblivious as sko
    from parla.drivers.least_squares import SPO, SSO1
    A, b = _ls_problem(400, 20, 6, 1e-6, 41)
    out = {'A': A, 'b': b}
    gens = {'ga': sko.SkOpGA(), 'sj': sko.SkOpSJ(8), 'tc': sko.SkOpTC()}
    seed = 100
    for gname, gen in gens.items():
        for mode in ('qr', 'chol', 'svd'):
            seed += 1
            alg = SPO(gen, 4, mode)
            x, log = alg(A, b, 0.0, 1e-12, 100, np.random.default_rng(seed))
            out[f'{gname}_{mode}_seed'] = np.array(seed)
            out[f'{gname}_{mode}_x'] = x
            out[f'{gname}_{mode}_errors'] = log.errors
    x, log = SPO(sko.SkOpGA(), 3, 'qr')(A, b, 0.25, 1e-12, 100,
                                         np.random.default_rng(7))
    out['ridge_x'], out['ridge_errors'] = x, log.errors
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        x, _ = SSO1(sko.SkOpSJ(8), 3, 'gelsd')(A, b, 0.0, np.nan, 1,
                                               np.random.default_rng(9))
    out['sso_x'] = x
    return out


def spu_cases(parla):
    """SPU1 (underdetermined LS) as the reference's own tests set it up:
    A = U diag(spectrum) V' of full column rank, c = A' y0."""
    import parla.comps.sketchers.oblivious as sko
    import parla.utils.sketching as usk
    from parla.drivers.least_squares import SPU1
    out = {}
    for tag, (m, n, kind, cond, gen, seed) in {
            'lin': (300, 30, 'lin', 1e5, 'sj', 51),
            'log': (400, 25, 'log', 1e5, 'ga', 52),
            'tight': (200, 20, 'lin', 1e3, 'sj', 53)}.items():
        rng = np.random.default_rng(seed)
        if kind == 'lin':
            spec = np.linspace(cond ** 0.5, cond ** -0.5, num=n)
        else:
            spec = np.logspace(np.log10(cond) / 2, -np.log10(cond) / 2, num=n)
        U = usk.orthonormal_operator(m, n, rng)
        Vt = usk.orthonormal_operator(n, n, rng)
        A = (U * spec) @ Vt
        c = A.T @ rng.standard_normal(m)
        alg = SPU1(sko.SkOpSJ(8) if gen == 'sj' else sko.SkOpGA(), 3)
        tol, lim = (0.0, n) if tag == 'tight' else (1e-12, 50)
        y, log = alg(A, c, tol, lim, np.random.default_rng(seed + 100))
        out[f'{tag}_A'], out[f'{tag}_c'] = A, c
        out[f'{tag}_gen'] = np.array(gen)
        out[f'{tag}_seed'] = np.array(seed + 100)
        out[f'{tag}_tol'], out[f'{tag}_lim'] = np.array(tol), np.array(lim)
        out[f'{tag}_y'], out[f'{tag}_errors'] = y, log.errors
    return out


def _saddle_problem(m, n, spec, delta, seed):
    """A = U diag(spec) V' (full column rank); b 70 % in range(A); c ~ N(0, I)."""
    import parla.utils.sketching as usk
    rng = np.random.default_rng(seed)
    U = usk.orthonormal_operator(m, n, rng)
    Vt = usk.orthonormal_operator(n, n, rng)
    A = (U * spec) @ Vt
    b0 = rng.standard_normal(m)
    br = U @ (U.T @ b0)
    bo = b0 - br
    b = 0.7 * br * (np.mean(spec) / np.linalg.norm(br)) + 0.3 * bo * (np.mean(spec) / np.linalg.norm(bo))
    c = rng.standard_normal(n)
    return A, b, c


def sps_cases(parla):
    """SPS1 (PCG; full-rank and both Nystrom strategies) and SPS2 (LSQR)."""
    import parla.comps.sketchers.oblivious as sko
    from parla.drivers.saddlesys import SPS1, SPS2
    out = {}
    cases = {
        'full0': ('sps1', 'ga', 3, 'left', 0.0, 61),
        'full5': ('sps1', 'sj', 3, 'left', 0.5, 62),
        'left': ('sps1', 'ga', 0.5, 'left', 0.5, 63),
        'right': ('sps1', 'ga', 0.5, 'right', 0.5, 64),
        'two0': ('sps2', 'sj', 3, None, 0.0, 65),
        'two1': ('sps2', 'ga', 3, None, 1.0, 66),
    }
    for tag, (alg_name, gen, sf, strat, delta, seed) in cases.items():
        A, b, c = _saddle_problem(300, 30, np.linspace(1e2, 1e-2, 30), delta, seed)
        op = sko.SkOpSJ(8) if gen == 'sj' else sko.SkOpGA()
        if alg_name == 'sps1':
            alg = SPS1(op, sf, None)
            alg.nystrom_strategy = strat
            tol = 1e-12
        else:
            alg = SPS2(op, sf, None)
            tol = 1e-12
        x, y, log = alg(A, b, c, delta, tol, 100, np.random.default_rng(seed + 100), logging=True)
        for k, v in (('A', A), ('b', b), ('c', c), ('x', x), ('y', y), ('errors', log.errors)):
            out[f'{tag}_{k}'] = v
        out[f'{tag}_meta'] = np.array(repr(dict(alg=alg_name, gen=gen, sf=sf, strategy=strat, delta=delta,
                                                seed=seed + 100, tol=tol, iter_lim=100)))
    return out


def lowrank_cases(parla):
    import parla.comps.sketchers.oblivious as sko
    from parla.comps.sketchers.aware import RS1
    from parla.comps.rangefinders import RF1
    from parla.comps.qb import QB1, QB2, QB3
    from parla.drivers.svd import SVD1
    from parla.drivers.evd import EVD1, EVD2
    import parla.utils.linalg_wrappers as law
    rng = np.random.default_rng(51)
    m, n = 120, 60
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.arange(1, n + 1, dtype=float) ** -1.5 + 1e-3
    A = (U * s) @ V.T
    out = {'A': A}
    for p in range(4):
        rs = RS1(sko.SkOpGA(), p, law.orth, 1)
        out[f'rs1_p{p}'] = rs(A, 10, np.random.default_rng(60 + p))
    rs = RS1(sko.SkOpGA(), 4, law.orth, 2)
    out['rs1_p4_s2'] = rs(A, 10, np.random.default_rng(65))
    rf = RF1(RS1(sko.SkOpGA(), 2, law.orth, 1))
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        out['rf1_Q'] = rf(A, 12, np.nan, np.random.default_rng(70))
    qb = QB1(rf)
    out['qb1_Q'], out['qb1_B'] = qb(A, 12, np.nan, np.random.default_rng(71))
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        rf0 = RF1(RS1(sko.SkOpGA(), 2, law.orth, 1))
        out['qb2_Q'], out['qb2_B'] = QB2(rf0, 5, False)(A, 17, 0.0, np.random.default_rng(76))
        out['qb2t_Q'], out['qb2t_B'] = QB2(rf0, 4, False)(A, 40, 0.05, np.random.default_rng(77))
        out['qb3_Q'], out['qb3_B'] = QB3(RS1(sko.SkOpGA(), 2, law.orth, 1), 5)(A, 17, 0.0,
                                                                            np.random.default_rng(78))
        out['qb3t_Q'], out['qb3t_B'] = QB3(RS1(sko.SkOpGA(), 2, law.orth, 1), 4)(A, 40, 0.05,
                                                                             np.random.default_rng(79))
        U1, s1, Vh1 = SVD1(qb)(A, 10, np.nan, 5, np.random.default_rng(72))
    out['svd1_U'], out['svd1_s'], out['svd1_Vh'] = U1, s1, Vh1
    # symmetric and PSD inputs for the eigensolvers
    W, _ = np.linalg.qr(rng.standard_normal((80, 80)))
    lam = np.linspace(1, 80, 80) ** -1.0 * np.where(np.arange(80) % 3 == 0, -1, 1)
    Asym = (W * lam) @ W.T
    Asym = 0.5 * (Asym + Asym.T)
    out['Asym'] = Asym
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        V1, l1 = EVD1(qb)(Asym, 10, np.nan, 4, np.random.default_rng(73))
    out['evd1_V'], out['evd1_lamb'] = V1, l1
    lam_psd = np.exp(-np.arange(80) / 6.0)
    Apsd = (W * lam_psd) @ W.T
    Apsd = 0.5 * (Apsd + Apsd.T)
    out['Apsd'] = Apsd
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        V2, l2 = EVD2(RS1(sko.SkOpGA(), 0, law.orth, 1))(Apsd, 12, np.nan, 4,
                                                         np.random.default_rng(74))
        V3, l3 = EVD2(RS1(sko.SkOpGA(), 2, law.orth, 1))(Apsd, 12, np.nan, 4,
                                                         np.random.default_rng(75))
    out['evd2_V'], out['evd2_lamb'] = V2, l2
    out['evd2p2_V'], out['evd2p2_lamb'] = V3, l3
    return out


def ls_fixtures(parla):
    """SHA-256 digests of the reference test suite's least-squares problems.

    The builders live in the reference's test module
    (parla/tests/test_drivers/test_optim/test_overdet_least_squares.py:11-108);
    the arrays are large, so only digests of A and b and the small x_opt are
    kept.  ``tests/lsfixtures.py`` restates the builders and must match.
    """
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tests.lsfixtures import digest
    import importlib
    mod = importlib.import_module('parla.tests.test_drivers.test_optim.test_overdet_least_squares')
    out = {}
    for name in ('consistent_tall', 'consistent_lowrank', 'consistent_square', 'inconsistent_orthog',
                 'inconsistent_gen', 'inconsistent_stackid'):
        ath = getattr(mod, name)()
        out[f'{name}_A'] = digest(ath.A)
        out[f'{name}_b'] = digest(ath.b)
        out[f'{name}_x'] = np.asarray(ath.x_opt, dtype=np.float64)
    return out


# (m, n, rank, k, over, axis, seed) of the reference's OSID tests
# (parla/tests/test_drivers/test_lowrank/test_osid.py:51-81), num_pass 0 / 2
OSID_CASES = {0: [(100, 30, 29, 29, 0, 0, 0), (100, 30, 28, 28, 1, 0, 2), (100, 30, 3, 3, 0, 0, 2),
                  (100, 30, 29, 29, 0, 1, 0), (100, 30, 28, 28, 1, 1, 2), (100, 30, 3, 3, 2, 1, 2)],
              2: [(100, 30, 30, 27, 3, 0, 0), (100, 30, 30, 25, 4, 0, 0), (100, 30, 30, 5, 5, 0, 0),
                  (30, 100, 30, 27, 3, 1, 0), (30, 100, 30, 25, 4, 1, 0), (30, 100, 30, 5, 5, 0, 0)]}
# (m, n, rank, k, over, seed) of the TSID tests (test_tsid.py:41-80)
TSID_CASES = {0: [(1000, 300, 290, 290, 0, 0), (1000, 300, 290, 290, 5, 2), (1000, 300, 30, 30, 0, 2),
                  (300, 1000, 290, 290, 0, 0), (300, 1000, 290, 290, 5, 2), (300, 1000, 30, 30, 0, 2)],
              2: [(100, 30, 30, 27, 3, 0), (100, 30, 30, 25, 4, 0), (30, 100, 30, 27, 3, 0),
                  (30, 100, 30, 25, 4, 0)]}
# (m, n, rank, k, over, seed) of the CUR tests (test_cur.py:34-75), num_pass 0 / 4
CUR_CASES = {0: [(100, 30, 24, 25, 3, 0), (100, 30, 5, 5, 1, 2), (30, 100, 24, 25, 3, 0), (30, 100, 5, 5, 1, 2)],
             4: [(100, 30, 30, 27, 3, 0), (100, 30, 30, 25, 4, 0), (100, 30, 30, 5, 5, 0),
                 (30, 100, 30, 27, 3, 0), (30, 100, 30, 25, 4, 0), (30, 100, 30, 5, 5, 0)]}


def interp_cases(parla):
    """Outputs of the reference's interpolative decompositions on its own test
    configurations: the matrix comes from rand_low_rank(m, n, rank, rng) and
    the algorithm continues the same Generator, as in the reference's tests.
    Large coefficient matrices are stored as fingerprints (products with a
    fixed Gaussian vector) next to their digests."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tests.lsfixtures import digest
    import parla.tests.matmakers as mm
    import parla.comps.sketchers.oblivious as obl
    import parla.utils.linalg_wrappers as ulaw
    from parla.comps.sketchers.aware import RS1
    from parla.drivers.interpolative import OSID1, OSID2, TSID1, CUR1
    from parla.comps.interpolative import ROCS1, qrcp_osid
    out = {}

    def rs(p):
        return RS1(sketch_op_gen=obl.SkOpGA(), num_pass=p, stabilizer=ulaw.orth, passes_per_stab=1)

    def keep(tag, M):
        M = np.asarray(M, dtype=np.float64)
        if M.size <= 4000:
            out[tag] = M
        else:
            g = np.random.default_rng(99).standard_normal(M.shape[1])
            out[tag + '_fp'] = M @ g
            out[tag + '_digest'] = digest(M)

    for p, cases in OSID_CASES.items():
        for ci, (m, n, rank, k, over, axis, seed) in enumerate(cases):
            for an, cls in (('osid1', OSID1), ('osid2', OSID2)):
                rng = np.random.default_rng(seed)
                A = mm.rand_low_rank(m, n, rank, rng)
                M, P = cls(rs(p))(A, k, over, axis, rng)
                tag = f'{an}_p{p}_{ci}'
                out[tag + '_A'] = digest(A)
                keep(tag + '_M', M)
                out[tag + '_P'] = np.asarray(P, dtype=np.int64)
    for p, cases in TSID_CASES.items():
        for ci, (m, n, rank, k, over, seed) in enumerate(cases):
            rng = np.random.default_rng(seed)
            A = mm.rand_low_rank(m, n, rank, rng)
            Z, I, X, J = TSID1(OSID1(rs(p)))(A, k, over, rng)
            tag = f'tsid1_p{p}_{ci}'
            out[tag + '_A'] = digest(A)
            keep(tag + '_Z', Z)
            keep(tag + '_X', X)
            out[tag + '_I'] = np.asarray(I, dtype=np.int64)
            out[tag + '_J'] = np.asarray(J, dtype=np.int64)
    for p, cases in CUR_CASES.items():
        for ci, (m, n, rank, k, over, seed) in enumerate(cases):
            rng = np.random.default_rng(seed)
            A = mm.rand_low_rank(m, n, rank, rng)
            Js, U, Is = CUR1(OSID1(rs(p)))(A, k, over, rng)
            tag = f'cur1_p{p}_{ci}'
            out[tag + '_A'] = digest(A)
            keep(tag + '_U', U)
            out[tag + '_Js'] = np.asarray(Js, dtype=np.int64)
            out[tag + '_Is'] = np.asarray(Is, dtype=np.int64)
    for ci, (axis, p) in enumerate(((0, 2), (1, 2), (0, 0))):
        rng = np.random.default_rng(40 + ci)
        A = mm.rand_low_rank(120, 80, 40, rng)
        out[f'rocs1_{ci}_A'] = digest(A)
        out[f'rocs1_{ci}_idx'] = np.asarray(ROCS1(rs(p))(A, 20, 5, axis, rng), dtype=np.int64)
    Y = np.random.default_rng(50).standard_normal((30, 90))
    for axis in (0, 1):
        M, P = qrcp_osid(Y if axis == 1 else Y.T, 20, axis)
        out[f'qrcp_osid_{axis}_M'] = M
        out[f'qrcp_osid_{axis}_P'] = np.asarray(P, dtype=np.int64)
    return out


def main(ref_path, only=None):
    """Write every fixture, or only those named in ``only``."""
    parla = _import_reference(ref_path)
    meta = dict(numpy=np.__version__, scipy=scipy.__version__,
                parla=parla.__version__)
    for name, fn in (('sketch', sketches), ('lsqr', lsqr_case),
                     ('spo', spo_cases), ('spu', spu_cases), ('sps', sps_cases),
                     ('lowrank', lowrank_cases), ('lsfix', ls_fixtures), ('interp', interp_cases)):
        if only and name not in only:
            continue
        data = fn(parla)
        data['_versions'] = np.array(repr(meta))
        path = os.path.join(HERE, f'{name}.npz')
        np.savez_compressed(path, **data)
        print('wrote', path, sum(v.nbytes for v in data.values()), 'bytes')


if __name__ == '__main__':
    if len(sys.argv) < 2:
        sys.exit('usage: make_golden.py <path to the reference source tree> [fixture names ...]')
    main(sys.argv[1], sys.argv[2:])
