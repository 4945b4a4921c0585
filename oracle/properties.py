"""Test infrastructure: restatement of the reference's brute-force one-particle
density matrix of an MPS (``properties/mpo_dmrg_propsItrf.eval_rdm1BF``,
mpo_dmrg_propsItrf.py:204-263, the non-spin-projected branch), with the
pieces it calls:

* ``genMPO_Epq`` (``properties/mpo_dmrg_propsMPO.py``, genMPO_Epq): two
  operators, E_pq^alpha = a+_{2p} a_{2q} and E_pq^beta = a+_{2p+1} a_{2q+1},
  each a bond-dimension-1 MPO whose site tensors are the products of the
  elementary spatial operators (``mpo_dmrg_opers.genElemProductSpatial``,
  mpo_dmrg_opers.py:83-88: Jordan-Wigner string left of the orbital,
  creation / annihilation on it, identity right of it);
* ``evalPropsNQt`` (``properties/mpo_dmrg_props.py:39-86``, status 'L'): the
  left environments <bra|O|ket> site by site, with the reference's three
  tensordots, and the expectation value at the last site.

Dense (NQt) site tensors [left bond, local state, right bond] of a
left-canonical MPS; the last site carries the normalised state.  Only the
tests use this module.
"""
import numpy

from .mpo import genElemSpatialMat


def genElemProductSpatial(oplst, isite):
    """[[p, iop], ...] -> the product of the elementary operators on ``isite``
    as a (1, 1, 4, 4) MPO site (mpo_dmrg_opers.py:83-88)."""
    p0, iop0 = oplst[0]
    mat = genElemSpatialMat(p0, isite, iop0)
    for p1, iop1 in oplst[1:]:
        mat = mat.dot(genElemSpatialMat(p1, isite, iop1))
    return mat.reshape(1, 1, 4, 4)


def genMPO_Epq(nsite, p, q):
    """Site tensors of E_pq^alpha and E_pq^beta: ops[isite][iop]."""
    return [[genElemProductSpatial([[2 * p + s, 1], [2 * q + s, 0]], isite) for s in (0, 1)]
            for isite in range(nsite)]


def evalPropsNQt(bra, ket, ops):
    """<bra|O_iop|ket> for every operator of ``ops`` (left sweep)."""
    nsite = len(ket)
    nop = len(ops[0])
    envs = [numpy.ones((1, 1, 1)) for _ in range(nop)]
    for isite in range(nsite):
        for iop in range(nop):
            cop = ops[isite][iop]
            tmp = numpy.tensordot(bra[isite].conj(), envs[iop], axes=([0], [1]))
            tmp = numpy.tensordot(cop, tmp, axes=([0, 2], [2, 0]))
            tmp = numpy.tensordot(tmp, ket[isite], axes=([1, 3], [1, 0]))
            envs[iop] = tmp
    return numpy.array([e[0, 0, 0] for e in envs])


def eval_rdm1BF(sites):
    """(rdm1t, rdm1s): spin-summed and spin (0.5 (alpha - beta)) one-particle
    density matrices of the MPS, element by element as the reference does."""
    nsite = len(sites)
    rdm1 = numpy.zeros((nsite, nsite, 2))
    for p in range(nsite):
        for q in range(nsite):
            if p > q:
                continue
            exphop = evalPropsNQt(sites, sites, genMPO_Epq(nsite, p, q))
            rdm1[p, q] = exphop
            rdm1[q, p] = exphop
    rdm1 = rdm1.transpose(2, 0, 1)
    rdm1t = rdm1[0] + rdm1[1]
    rdm1s = 0.5 * (rdm1[0] - rdm1[1])
    assert numpy.linalg.norm(rdm1t - rdm1t.T) < 1e-12
    assert numpy.linalg.norm(rdm1s - rdm1s.T) < 1e-12
    return rdm1t, rdm1s


def mps_to_fock(sites):
    """The state vector of a dense MPS in the Fock basis of the
    Jordan-Wigner operators of ``integrals`` (spin-orbitals 2i, 2i+1 of
    spatial site i, the first one most significant)."""
    v = numpy.ones((1, 1))
    for t in sites:
        v = numpy.tensordot(v, t, axes=([1], [0]))
        v = v.reshape(-1, t.shape[2])
    return v.reshape(-1)
