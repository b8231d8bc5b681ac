/*
 * ref_ensobs.c -- the reference's own calc/ensobs.c, compiled unmodified
 * inside this translation unit.  TEST INFRASTRUCTURE ONLY:
 * oracle/_ref/libenkf_ref_ensobs.so pins the oracle's restatement of
 * das_calcinnandspread (calc/ensobs.c:541-690) and das_standardise
 * (calc/ensobs.c:849-898) against the reference itself.
 *
 * The entry points below build the reference's own dasystem and
 * observations structures in memory (the fields these two functions read:
 * the ensemble S, the observations' value, status, estd and type, the
 * types' rfactor) and call the functions as the reference's enkf_calc does.
 * The rest of ensobs.c (HE from the model fields, file output) names the
 * model, grid, NetCDF and observation modules; ref_ensobs_stubs.c defines
 * those to abort if reached.
 */
#include "ensobs.c"

/* das_calcinnandspread on S [nmem][nobs] (HE in, HA out, in place): the
 * innovations s_f and spreads std_f [nobs] come back */
int ref_calcinnandspread(int nmem, int nobs, float* S, const float* value, const short* status, double* s_f,
                         double* std_f)
{
    dasystem das;
    observations obs;
    observation* data = calloc(nobs > 0 ? nobs : 1, sizeof(observation));
    float** rows = malloc((nmem > 0 ? nmem : 1) * sizeof(float*));
    int e, o;

    memset(&das, 0, sizeof(das));
    memset(&obs, 0, sizeof(obs));
    for (o = 0; o < nobs; ++o) {
        data[o].id = o;
        data[o].value = value[o];
        data[o].status = status[o];
    }
    obs.nobs = nobs;
    obs.data = data;
    for (e = 0; e < nmem; ++e)
        rows[e] = S + (size_t) e * nobs;
    das.nmem = nmem;
    das.S = rows;
    das.obs = &obs;
    das.s_mode = S_MODE_HE_f;
    das_calcinnandspread(&das);
    if (nobs > 0) {
        memcpy(s_f, das.s_f, nobs * sizeof(double));
        memcpy(std_f, das.std_f, nobs * sizeof(double));
    }
    free(das.s_f);
    free(das.std_f);
    free(rows);
    free(data);
    return 0;
}

/* das_standardise on S [nmem][nobs] and s_f [nobs] (HA and innovations in,
 * standardised out, in place), with the observations' estd and type and the
 * types' rfactor [ntypes] */
int ref_standardise(int nmem, int nobs, float* S, double* s_f, const float* estd, const short* type, int ntypes,
                    const double* rfactor)
{
    dasystem das;
    observations obs;
    observation* data = calloc(nobs > 0 ? nobs : 1, sizeof(observation));
    obstype* types = calloc(ntypes > 0 ? ntypes : 1, sizeof(obstype));
    float** rows = malloc((nmem > 0 ? nmem : 1) * sizeof(float*));
    int e, o, t;

    memset(&das, 0, sizeof(das));
    memset(&obs, 0, sizeof(obs));
    for (o = 0; o < nobs; ++o) {
        data[o].id = o;
        data[o].estd = estd[o];
        data[o].type = type[o];
    }
    for (t = 0; t < ntypes; ++t)
        types[t].rfactor = rfactor[t];
    obs.nobs = nobs;
    obs.data = data;
    obs.nobstypes = ntypes;
    obs.obstypes = types;
    for (e = 0; e < nmem; ++e)
        rows[e] = S + (size_t) e * nobs;
    das.nmem = nmem;
    das.S = rows;
    das.s_f = s_f;
    das.obs = &obs;
    das.s_mode = S_MODE_HA_f;
    das_standardise(&das);
    free(rows);
    free(types);
    free(data);
    return 0;
}
