"""Optical configurations of the PSF-generation golden vectors (small, seconds each).

Each case gives the arguments of GeneratePSF (reference generate_psf.py:63);
lengths in metres.  Shared by the fixture generator (which runs the
reference's generator) and the tests.
"""

PSF_CASES = {
    # M40 / NA 0.95 water objective optics of the light-field literature, Nnum 5, 5 planes incl. z = 0
    "n5_osr3": dict(M=40, NA=0.95, MLPitch=150e-6, Nnum=5, OSR=3, n=1.33, fml=3000e-6, lam=520e-9,
                    zmin=-6e-6, zmax=6e-6, zspacing=3e-6, normalisePSF=True, reproduceMaxBug=False),
    # a deeper z range: PSF sizes differ per plane, so CAindex crops
    "n7_z30": dict(M=40, NA=0.95, MLPitch=150e-6, Nnum=7, OSR=3, n=1.33, fml=3000e-6, lam=520e-9,
                   zmin=-30e-6, zmax=30e-6, zspacing=10e-6, normalisePSF=True, reproduceMaxBug=False),
    # lower NA, Nnum 7, un-normalised with the reference's reproduced z = 0 maximum bug
    "n7_bug": dict(M=20, NA=0.5, MLPitch=125e-6, Nnum=7, OSR=3, n=1.0, fml=2500e-6, lam=520e-9,
                   zmin=-10e-6, zmax=10e-6, zspacing=10e-6, normalisePSF=False, reproduceMaxBug=True),
}
