"""Reduced density matrices of an MPS through the MPO environments.

The reference evaluates the spin-summed one-particle density matrix by
brute force over MPOs of E_pq (``properties/mpo_dmrg_propsItrf.eval_rdm1BF``,
mpo_dmrg_propsItrf.py:204-263) and two-particle elements with
``genMPO_Apqrs`` + ``evalProps`` (``properties/mpo_dmrg_propsMPO.py:73-113``).
Here both come from one pass of site gradients of the Hamiltonian MPO
(``adjoint.site_gradients``): the energy functional <psi|H(h, g)|psi> is
linear in the integrals, so

    gamma[p, q] = d<H>/d h1e[p, q]          = sum_s <a+_ps a_qs>
    Gamma[p, q, r, s] = 2 d<H>/d (pq|rs)    = sum_st <a+_ps a+_rt a_st a_qs>

for any MPS (not only a converged one), with the environments, site
gradients and chain rule of the gradient code.
"""
from . import adjoint


def rdm12(dmrg, h1e, eri, fmps=None):
    """(gamma, Gamma) of the MPS ``fmps`` (default: the driver's last
    left-canonical MPS).  ``h1e``, ``eri``: the spatial integrals the driver's
    MPO was built from (any values: the densities do not depend on them)."""
    grads, _, _ = adjoint.site_gradients(dmrg, fmps)
    dh, dg = adjoint.integral_gradients(dmrg, h1e, eri, grads)
    return dh, 2.0 * dg


def rdm1(dmrg, h1e, eri, fmps=None):
    """Spin-summed one-particle density matrix gamma[p, q] = <E_pq>."""
    return rdm12(dmrg, h1e, eri, fmps)[0]
