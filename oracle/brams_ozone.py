"""Scalar restatement of BRAMS's ozone climatology for the radiation columns
-- TEST INFRASTRUCTURE ONLY.

Follows src/brams/radiate/rtm_driver.f90 statement by statement, in plain
Python loops with 1-based subscripts: the column's sigma levels (:1120-1140),
InitGetoz_rrtm's per-column set-up (:2619-2634; year_getoz and mon_getoz are
INTEGER variables, so 365.25 and 365.25/12 are stored as 365 and 30),
getoz_rrtm (:2638-2823) and the flip into o3vmr without chemistry ozone
(:1168-1173).  The table is ``ozone(18, 37, 4)`` / ``ozsig(18)`` of
brams_ozone.gblw.  The product library never uses this file.
"""
from __future__ import annotations

import math

PAI = 3.1415926e0
RLAG = 14.8125e0
YEAR, MON = 365, 30
RO3AR = 1 / (47.998e0 / 28.96e0)


def getoz(ozone, ozsig, kmax, sigmid, colrad, date, inter):
    """o3l(1..kmax) as a 0-based list; sigmid is 1-based (index 0 unused)."""
    oz = lambda k, la, s: float(ozone[k - 1, la - 1, s - 1])
    zs = lambda k: float(ozsig[k - 1])
    if date > YEAR:
        date = date - YEAR
    imon = int(date / MON + 1)
    if imon < 1:
        imon = 1
    isea = imon // 3 + 1
    if isea == 5:
        isea = 1
    if isea > 5:
        raise ValueError("ERROR IN ISEA")
    theta = 90.0 - (180.0 / PAI) * colrad
    flat = 0.2 * theta
    la = int(19.501e0 - flat)
    ll = int(19.001e0 - flat)
    rang = 2.0e0 * PAI * (date - RLAG) / YEAR
    rsin1, rcos1, rcos2 = math.sin(rang), math.cos(rang), math.cos(2.0e0 * rang)
    rate = float(19 - ll) - flat
    ozo3l = [0.0] * 19
    for k in range(1, 19):
        a1 = 2.5e-1 * (oz(k, la, 1) + oz(k, la, 2) + oz(k, la, 3) + oz(k, la, 4))
        a2 = 0.5e0 * (oz(k, la, 2) - oz(k, la, 4))
        a3 = 0.5e0 * (oz(k, la, 1) - oz(k, la, 3))
        a4 = 2.5e-1 * (oz(k, la, 1) + oz(k, la, 3) - oz(k, la, 2) - oz(k, la, 4))
        b1 = 2.5e-1 * (oz(k, ll, 1) + oz(k, ll, 2) + oz(k, ll, 3) + oz(k, ll, 4))
        b2 = 0.5e0 * (oz(k, ll, 2) - oz(k, ll, 4))
        b3 = 0.5e0 * (oz(k, ll, 1) - oz(k, ll, 3))
        b4 = 2.5e-1 * (oz(k, ll, 1) + oz(k, ll, 3) - oz(k, ll, 2) - oz(k, ll, 4))
        do3a = a1 + rsin1 * a2 + rcos1 * a3 + rcos2 * a4
        do3b = b1 + rsin1 * b2 + rcos1 * b3 + rcos2 * b4
        ozo3l[k] = do3a + rate * (do3b - do3a)
        ozo3l[k] = 1.0e-04 * ozo3l[k]
    o3l = [0.0] * max(kmax, 18)
    if inter:
        kk = [0] * (kmax + 1)
        notfound = [False] * (kmax + 1)
        for l in range(1, kmax + 1):
            notfound[l] = sigmid[l] > zs(1)
            kk[l] = 18 if notfound[l] else 2
        for l in range(1, kmax + 1):
            if notfound[l]:
                for k in range(2, 19):
                    if sigmid[l] > zs(k - 1) and sigmid[l] <= zs(k):
                        kk[l] = k
                        break
        for l in range(1, kmax + 1):
            aa = (ozo3l[kk[l]] - ozo3l[kk[l] - 1]) / (zs(kk[l]) - zs(kk[l] - 1))
            bb = ozo3l[kk[l] - 1] - aa * zs(kk[l] - 1)
            o3l[kmax + 1 - l - 1] = bb + aa * sigmid[l]
    else:
        for l in range(1, 19):
            o3l[l - 1] = ozo3l[l]
    return o3l


def o3vmr_columns(ozone, ozsig, plev, glat, doy):
    """plev (ncol, mzp) interface pressures, glat (ncol,) float32 degrees ->
    o3vmr (ncol, mzp - 1) as radrrtmdrv forms it."""
    ncol, mzp = plev.shape
    out = [[0.0] * (mzp - 1) for _ in range(ncol)]
    for noc in range(ncol):
        sig = [0.0] * (mzp + 2)
        for i in range(2, mzp + 1):
            sig[i] = float(plev[noc, i - 1]) / float(plev[noc, 0])
        sig[1] = 1.0
        sig[mzp + 1] = 0.0
        sigmid = [0.0] * (mzp + 2)
        for k in range(1, mzp + 1):
            sigmid[k] = (sig[k] + sig[k + 1]) / 2
        inter = 18 != mzp
        if not inter:
            for l in range(1, 19):
                if abs(float(ozsig[l - 1]) - sig[18 - l + 1]) > 0.0001:
                    inter = True
        colrad = PAI * (1.00e0 - (float(glat[noc]) + 90.00e0) / 180.00e0)
        o3l = getoz(ozone, ozsig, mzp, sigmid, colrad, float(doy), inter)
        for k in range(1, mzp):
            out[noc][k - 1] = o3l[mzp + 1 - k - 1] * RO3AR
    return out
