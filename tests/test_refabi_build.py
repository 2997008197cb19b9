"""CPU test of refabi.build: the reference-layout structs (Params, Track2D,
Track, Source; src/SimpleMOC_header.h:86-158) it fills through numpy views are
read back through ctypes, the way the reference's code dereferences them."""
import numpy as np


def test_reference_structs_point_at_the_problem_arrays(lib):
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import refabi
    spec = sm.ProblemSpec(n_groups=9, fai=5, cai=4, height=40.0, n_sources=37, n_tracks_2d=5,
                          n_polar=4, z_stacked=80, n_seg=10, n_materials=6, seed=3)
    hp = sm.generate(spec)
    geo = refabi.make_geometry(4, 5, 4, 80, 12, 0.5)
    rp = refabi.build(hp, geo)
    G, F, P, Z = spec.n_groups, spec.fai, spec.n_polar, 80
    prm = rp.params
    rng = np.random.default_rng(0)
    # 2D tracks and their segments
    for i in range(5):
        t2 = prm.tracks_2D[i]
        n = int(geo.seg_off[i + 1] - geo.seg_off[i])
        assert t2.n_segments == n and t2.az_weight == np.float32(geo.az_weight[i])
        for s in range(n):
            assert t2.segments[s].length == geo.seg_len[geo.seg_off[i] + s]
    # 3D tracks: tracks[i][j][k]
    for _ in range(50):
        i, j, k = int(rng.integers(5)), int(rng.integers(P)), int(rng.integers(Z))
        t = (i * P + j) * Z + k
        tr = prm.tracks[i][j][k]
        assert tr.p_weight == geo.p_weight[t] and tr.z_height == geo.z_height[t]
        g = int(rng.integers(G))
        rp.psi_f[t * G + g] = 1.5 + t
        rp.psi_b[t * G + g] = -2.5 - t
        assert tr.f_psi[g] == np.float32(1.5 + t) and tr.b_psi[g] == np.float32(-2.5 - t)
    # sources: fine rows, sigma_t row, cross sections and scatter of the material
    xs3 = hp.xs.reshape(-1, G, 3)
    sc = hp.scatter.reshape(-1, G, G)
    sig = hp.sigt.reshape(-1, G)
    for _ in range(50):
        n = int(rng.integers(spec.n_sources))
        src = prm.sources[n]
        f, g, g2 = int(rng.integers(F)), int(rng.integers(G)), int(rng.integers(G))
        assert src.fine_source[f][g] == rp.fine_source[(n * F + f) * G + g]
        rp.fine_flux[(n * F + f) * G + g] = 7.0 + n
        assert src.fine_flux[f][g] == np.float32(7.0 + n)
        assert src.vol == hp.vol[n]
        assert src.sigT[g] == sig[hp.src_sigt[n], g]
        m = int(hp.src_xs[n])
        assert [src.XS[g][c] for c in range(3)] == list(xs3[m, g])
        assert src.scattering_matrix[g][g2] == sc[m, g, g2]
    assert rp.input.ntracks == 5 * P * Z and rp.input.n_egroups == G
