/* Stand-in PAL prototypes for compiling the reference geometry.c in the
 * oracle harness. The harness never calls the functions that use them
 * (calc_beam_geom, mjd2lst, parse_ra/parse_dec); pal_stubs.c aborts if they
 * are reached. */
#ifndef VGB_STUB_PAL_H
#define VGB_STUB_PAL_H
void palMap(double rm, double dm, double pr, double pd, double px, double rv,
            double eq, double date, double *ra, double *da);
void palDe2h(double ha, double dec, double phi, double *az, double *el);
double palRanorm(double angle);
double palGmst(double ut1);
void palDtf2r(int ihour, int imin, double sec, double *rad, int *j);
void palDaf2r(int ideg, int iamin, double asec, double *rad, int *j);
void palCaldj(int iy, int im, int id, double *djm, int *j);
void palDh2e(double az, double el, double phi, double *ha, double *dec);
double palPa(double ha, double dec, double phi);
#endif
