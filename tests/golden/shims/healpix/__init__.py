"""Stand-in for ``healpix``: only pixel counts."""


def nside2npix(nside):
    return 12 * nside * nside


def npix2nside(npix):
    import math
    return int(math.isqrt(npix // 12))
