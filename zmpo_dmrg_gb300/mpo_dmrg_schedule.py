"""Sweep schedule (same interface as ``source/mpo_dmrg_schedule.py``):
``schedule(maxM, tol, maxiter)`` with ``normal(iop)`` / ``fixed(...)``,
``getParameters(dmrg, isweep)`` setting (ncsite, Dmax, crit_e, noise) and
``checkConv(dmrg, isweep, deltaE)``."""
import math


class schedule:
    TAGS = ('Normal0', 'Normal1', 'Normal2', 'Fixed1', 'Fixed2')

    def __init__(self, maxM=1000, tol=1.e-7, maxiter=40):
        self.maxM = maxM
        self.tol = tol
        self.maxiter = maxiter
        self.startM = None
        self.startTol = 1.e-4
        self.startNoise = 1.e-4
        self.coff = 2
        self.change = None
        self.Tag = None
        self.Sweeps, self.MaxMs, self.Tols, self.Noises = [], [], [], []

    def _set(self, dmrg, ncsite, idx):
        dmrg.ncsite = ncsite
        dmrg.status = 'twoSite' if ncsite == 2 else 'oneSite'
        dmrg.Dmax, dmrg.crit_e, dmrg.noise = self.MaxMs[idx], self.Tols[idx], self.Noises[idx]

    def getParameters(self, dmrg, isweep):
        if self.Tag not in self.TAGS:
            raise ValueError('no such Tag in taglst: %r' % (self.Tag,))
        last = len(self.MaxMs) - 1
        if self.Tag == 'Normal0':
            if isweep < self.change:
                self._set(dmrg, 2, min(last, isweep))
            else:
                self._set(dmrg, 1, last)
                if isweep == self.change:
                    dmrg.psi0 = None
        elif self.Tag in ('Normal1', 'Normal2'):
            self._set(dmrg, 1 if self.Tag == 'Normal1' else 2, min(last, isweep))
        else:
            self._set(dmrg, 1 if self.Tag == 'Fixed1' else 2, last)
        return 0

    def checkConv(self, dmrg, isweep, deltaE):
        if self.Tag.startswith('Normal'):
            return isweep > self.change and abs(deltaE) < self.tol
        return abs(deltaE) < self.tol

    def fixed(self, ncsite=2, maxM=None, tol=None, maxiter=None, noise=1.e-4):
        self.Tag = 'Fixed1' if ncsite == 1 else 'Fixed2'
        if maxM is not None:
            self.maxM = maxM
        if tol is not None:
            self.tol = tol
        if maxiter is not None:
            self.maxiter = maxiter
        self.Sweeps, self.MaxMs, self.Tols, self.Noises = [0], [self.maxM], [self.tol], [noise]
        self.change = 0
        return 0

    def normal(self, iop=0):
        self.Tag = ('Normal0', 'Normal1', 'Normal2')[iop]
        self.Sweeps, self.MaxMs, self.Tols, self.Noises = [], [], [], []
        if self.startM is None:
            self.startM = min(max(int(1.5 * math.sqrt(self.maxM)), 25), self.maxM)
        m = min(self.startM, self.maxM)
        n = 0
        tol, noise = self.startTol, self.startNoise
        while m < self.maxM:
            self.Sweeps.append(n)
            self.MaxMs.append(m)
            self.Tols.append(tol)
            self.Noises.append(noise)
            n += 1
            m *= 2
        first = True
        while tol >= self.tol:
            self.Sweeps.append(n)
            self.MaxMs.append(self.maxM)
            self.Tols.append(tol)
            self.Noises.append(noise)
            n += 1
            tol /= 10.0
            if first:
                noise = 0.0
                first = False
        self.change = n + self.coff
        return 0

    def collect(self):
        self.maxM = self.MaxMs[-1]
        self.tol = self.Tols[-1]
        self.change = self.Sweeps[-1] + 2
        self.maxiter = max(self.change, 40)
        return 0
