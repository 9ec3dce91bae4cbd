"""The two evaluations of the particle-particle ladder and of the t2 part of
the hole-hole intermediate that the engine's plan chooses between (site basis
for large molecules and FP64 iterations, MO basis for small molecules in
mixed precision) are the same numbers. Random orbitals, gamma, t1 and t2; no GPU.

  site:  sum_mu,nu X_mu,a X_nu,b gamma_mu,nu [sum_cd C_mu,c C_nu,d t_ij^cd]
  MO:    sum_cd (ac|bd)~ t_ij^cd,  (ac|bd)~ = sum_mu,nu X_mu,a Y_mu,c gamma X_nu,b Y_nu,d
  hole-hole: sum_mu,nu C_mu,k C_nu,l gamma_mu,nu Ts[i,mu,j,nu]  =  sum_cd (kc|ld) t_ij^cd
"""
import numpy as np


def test_site_and_mo_ladders_agree():
    rng = np.random.default_rng(7)
    N, o = 12, 5
    v = N - o
    C, _ = np.linalg.qr(rng.normal(size=(N, N)))
    g = rng.normal(size=(N, N)); g = g + g.T
    t1 = 0.1 * rng.normal(size=(o, v))
    t2 = 0.1 * rng.normal(size=(o, o, v, v))            # t2[i, j, a, b] = t_ij^ab
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))          # pair symmetry
    Co, Cv = C[:, :o], C[:, o:]
    X = np.hstack([Co, Cv - Co @ t1])                   # T1 dressing
    Y = np.hstack([Co + Cv @ t1.T, Cv])
    Xv, Yv = X[:, o:], Y[:, o:]
    assert np.array_equal(Yv, Cv) and np.array_equal(X[:, :o], Co)
    # site basis
    Ts = np.einsum("mc,nd,ijcd->imjn", Cv, Cv, t2) * g[None, :, None, :]
    lad_site = np.einsum("ma,nb,imjn->ijab", Xv, Xv, Ts)
    hh_site = np.einsum("mk,nl,imjn->klij", Co, Co, Ts)
    # MO basis
    Vvv = np.einsum("ma,mc,mn,nb,nd->acbd", Xv, Yv, g, Xv, Yv)
    lad_mo = np.einsum("acbd,ijcd->ijab", Vvv, t2)
    gov = np.einsum("mk,mc,mn,nl,nd->kcld", Co, Cv, g, Co, Cv)
    hh_mo = np.einsum("kcld,ijcd->klij", gov, t2)
    assert np.allclose(lad_site, lad_mo, rtol=1e-12, atol=1e-13)
    assert np.allclose(hh_site, hh_mo, rtol=1e-12, atol=1e-13)
