"""Empty stand-in for ``healpy``: the spherical-harmonic transform is patched in."""
