/*
 * ref_obs.c -- entry point into the reference's own common/observations.c
 * and common/obstypes.c (compiled unmodified, with common/kdtree.c,
 * common/hash.c and common/stringtable.c) for oracle/_ref/libenkf_ref_obs.so.
 * TEST INFRASTRUCTURE ONLY: pins the oracle's restatement of obs_findlocal
 * (common/observations.c:1837-1927: the type loop, domains, the status skip,
 * NLOBSMAX with the distance sort, the taper, obs_getglobal for a point
 * without coordinates) against the reference itself.
 *
 * The observation set is built in memory as the reference holds it after
 * reading and checking the observations: one obstype per type (radii,
 * weights, NLOBSMAX, the geographic flag, the domains it is visible from)
 * and one observation record per observation (position, type, status).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include "ncw.h"
#include "global.h"
#include "utils.h"
#include "observations.h"

/*
 * The observation set as the reference holds it after reading and checking
 * the observations: nobs records (lon, lat, type, status; value and estd
 * when given), ntypes types with nlocrad radii each (locrad, locweight
 * [ntypes][maxlocrad]), nlobsmax[t] (<= 0: no limit), visible[t] (NULL: all;
 * 0: the type's domain list names another domain than "grid"), the
 * geographic flag and rfactor[t] (NULL: 1).  Its kd-trees are built (so
 * that obs_getglobal finds the per-type ids they come with).
 */
observations* orref_obs_build(int nobs, const float* lon, const float* lat, const short* type, const short* status,
                              const float* value, const float* estd, int ntypes, int maxlocrad, const int* nlocrad,
                              const double* locrad, const double* locweight, const int* nlobsmax,
                              const int* visible, int geographic, const double* rfactor)
{
    static char* other[1] = { "other" };
    observations* obs = calloc(1, sizeof(observations));
    obstype* types = calloc(ntypes > 0 ? ntypes : 1, sizeof(obstype));
    observation* data = calloc(nobs > 0 ? nobs : 1, sizeof(observation));
    int t, o, k;

    for (t = 0; t < ntypes; ++t) {
        obstype* ot = &types[t];
        char name[32];

        snprintf(name, sizeof(name), "type%d", t);
        ot->id = t;
        ot->name = strdup(name);
        ot->nlocrad = nlocrad[t];
        ot->locrad = malloc(nlocrad[t] * sizeof(double));
        ot->locweight = malloc(nlocrad[t] * sizeof(double));
        for (k = 0; k < nlocrad[t]; ++k) {
            ot->locrad[k] = locrad[t * maxlocrad + k];
            ot->locweight[k] = locweight[t * maxlocrad + k];
        }
        ot->nlobsmax = (nlobsmax != NULL && nlobsmax[t] > 0) ? nlobsmax[t] : INT_MAX;
        ot->geographic = geographic;
        ot->rfactor = rfactor != NULL ? rfactor[t] : 1.0;
        if (visible != NULL && !visible[t]) {
            ot->ndomains = 1;
            ot->domainnames = other;
        }
    }
    for (o = 0; o < nobs; ++o) {
        data[o].id = o;
        data[o].lon = lon[o];
        data[o].lat = lat[o];
        data[o].type = type[o];
        data[o].status = status[o];
        if (value != NULL)
            data[o].value = value[o];
        if (estd != NULL)
            data[o].estd = estd[o];
        types[type[o]].nobs++;
    }
    obs->nobstypes = ntypes;
    obs->obstypes = types;
    obs->nobs = nobs;
    obs->data = data;
    obs_createkdtrees(obs);
    return obs;
}

void orref_obs_free(observations* obs)
{
    int t;

    obs_destroykdtrees(obs);
    if (obs->obsids != NULL) {
        for (t = 0; t < obs->nobstypes; ++t)
            free(obs->obsids[t]);
        free(obs->obsids);
    }
    for (t = 0; t < obs->nobstypes; ++t) {
        free(obs->obstypes[t].name);
        free(obs->obstypes[t].locrad);
        free(obs->obstypes[t].locweight);
    }
    free(obs->obstypes);
    free(obs->data);
    free(obs);
}

/*
 * obs_findlocal at nq queries (qlon, qlat; NaN: a point without
 * coordinates) of the set orref_obs_build makes.  Writes each query's count,
 * then its ids and taper coefficients one query after another in the
 * reference's order.  Returns the total count, or -1 if it exceeds cap.
 */
long long ref_findlocal(int nobs, const float* lon, const float* lat, const short* type, const short* status,
                        int ntypes, int maxlocrad, const int* nlocrad, const double* locrad,
                        const double* locweight, const int* nlobsmax, const int* visible, int geographic, int nq,
                        const double* qlon, const double* qlat, int* counts, int* ids, double* lcoeffs,
                        long long cap)
{
    observations* obs = orref_obs_build(nobs, lon, lat, type, status, NULL, NULL, ntypes, maxlocrad, nlocrad, locrad,
                                        locweight, nlobsmax, visible, geographic, NULL);
    long long total = 0;
    int k;

    for (k = 0; k < nq; ++k) {
        int n = 0, i;
        int* qids = NULL;
        double* qlc = NULL;

        obs_findlocal(obs, qlon[k], qlat[k], geographic, "grid", &n, &qids, &qlc, NULL);
        counts[k] = n;
        for (i = 0; i < n; ++i) {
            if (total + i < cap) {
                ids[total + i] = qids[i];
                lcoeffs[total + i] = qlc[i];
            }
        }
        total += n;
        free(qids);
        free(qlc);
    }
    orref_obs_free(obs);
    return total <= cap ? total : -1;
}
