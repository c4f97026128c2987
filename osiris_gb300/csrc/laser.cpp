// laser.cpp -- launch of a Gaussian laser pulse into the E and B arrays (host, once), as the
// reference's zpulse does at t = 0 for a forward-propagating pulse with a Gaussian longitudinal
// envelope and a Hermite-Gaussian TEM00 transverse profile:
//
//   field assignment      launch_zpulse_2d / launch_zpulse_3d, source/zpulse/os-zpulse-std.f03:
//                         1072-1212 / 1218-1390 (E2, E3 at the cell, B2, B3 half a cell ahead
//                         in x1, staggered transversely like the Yee grid; quadratic and
//                         quartic interpolation shift all positions by half a cell)
//   longitudinal          lon_envelope_zpulse, gaussian: exp(-2 ((x1 - x0) / duration)^2) for
//                         |x1 - x0| <= range / 2, else 0 (:2480-2561)
//   transverse            per_envelope_2d/3d_zpulse, hermite gaussian mode 0 (:2599-3049):
//                         sqrt(rWl2)^(dim - 1) / ... exp(-rho^2 rWl2 / w0^2)
//                         cos(k (x1 - x0) + k curv - gouy)
//   amplitude             omega0 * a0
//
// All arithmetic in double; the values are rounded to the field precision when stored.
#include <cmath>
#include <cstring>

#include "../../include/osiris_gb300.h"

namespace {

double lon_env(const osg_zpulse &z, double x)
{
    if (std::fabs(x - z.lon_x0) > z.lon_range / 2) return 0.0;
    const double s = (x - z.lon_x0) / z.lon_duration;
    return std::exp(-2 * (s * s));
}

// transverse envelope times the carrier at (x1, x2[, x3]) and t = 0
double per_env(const osg_zpulse &zp, int dim, double x1, double x2, double x3)
{
    const double k = zp.omega0;
    const double ox = x2 - zp.per_center[0], oy = dim > 2 ? x3 - zp.per_center[1] : 0.0;
    const double rho2 = dim > 2 ? ox * ox + oy * oy : ox * ox;
    const double z = x1 - zp.per_focus;
    const double z0 = dim > 2 ? k * (zp.per_w0 * zp.per_w0) / 2 : k * (zp.per_w0 * zp.per_w0) * 0.5;
    double rWl2 = 1, curv = 0, gouy = 0;
    if (z != 0) {
        rWl2 = (z0 * z0) / (z0 * z0 + z * z);
        curv = 0.5 * rho2 * z / (z * z + z0 * z0);
        gouy = std::atan2(z, z0);
    }
    const double amp = dim > 2 ? std::sqrt(rWl2) : std::sqrt(std::sqrt(rWl2));
    return amp * std::exp(-rho2 * rWl2 / (zp.per_w0 * zp.per_w0)) *
           std::cos(k * (x1 - zp.lon_x0) + k * curv - gouy);
}

template <typename T>
void launch(int dim, int order, const int *nx, const int *gcl, const int *gcu, const double *dx,
            const double *xmin, const osg_zpulse &zp, T *e, T *b)
{
    int size[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) size[d] = nx[d] + gcl[d] + gcu[d];
    const bool half = order == 2 || order == 4;
    const double zmin = xmin[0] + (half ? dx[0] / 2 : 0.0);
    const double r1min = xmin[1] + (half ? dx[1] / 2 : 0.0);
    const double r2min = dim > 2 ? xmin[2] + (half ? dx[2] / 2 : 0.0) : 0.0;
    const double cp = std::cos(zp.pol), sp = std::sin(zp.pol);
    const double amp = zp.omega0 * zp.a0;
    for (int j3 = 0; j3 < size[2]; j3++)
        for (int j2 = 0; j2 < size[1]; j2++)
            for (int j1 = 0; j1 < size[0]; j1++) {
                // Fortran cell index i = j - gcl + 1 (guard cells included)
                const int i1 = j1 - gcl[0] + 1, i2 = j2 - gcl[1] + 1;
                const int i3 = dim > 2 ? j3 - gcl[2] + 1 : 1;
                const double z = zmin + (double)(i1 - 1) * dx[0], z2 = z + dx[0] / 2;
                const double r1 = r1min + (double)(i2 - 1) * dx[1], r12 = r1 + dx[1] / 2;
                const double r2 = dim > 2 ? r2min + (double)(i3 - 1) * dx[2] : 0.0;
                const double r22 = dim > 2 ? r2 + dx[2] / 2 : 0.0;
                const double lenv = amp * lon_env(zp, z), lenv2 = amp * lon_env(zp, z2);
                const long p = 3L * (j1 + (long)size[0] * (j2 + (long)size[1] * j3));
                if (dim > 2) {
                    b[p + 1] = b[p + 1] - (T)(lenv2 * per_env(zp, 3, z2, r1, r22) * sp);
                    b[p + 2] = b[p + 2] + (T)(lenv2 * per_env(zp, 3, z2, r12, r2) * cp);
                    e[p + 1] = e[p + 1] + (T)(lenv * per_env(zp, 3, z, r12, r2) * cp);
                    e[p + 2] = e[p + 2] + (T)(lenv * per_env(zp, 3, z, r1, r22) * sp);
                } else {
                    b[p + 0] = (T)0;
                    b[p + 1] = (T)(-lenv2 * per_env(zp, 2, z2, r1, 0.0) * sp);
                    b[p + 2] = (T)(lenv2 * per_env(zp, 2, z2, r12, 0.0) * cp);
                    e[p + 0] = (T)0;
                    e[p + 1] = (T)(lenv * per_env(zp, 2, z, r12, 0.0) * cp);
                    e[p + 2] = (T)(lenv * per_env(zp, 2, z, r1, 0.0) * sp);
                }
            }
}

} // namespace

extern "C" int osg_zpulse_launch(int precision, int dim, int order, const int *nx,
                                 const int *gcl, const int *gcu, const double *dx,
                                 const double *xmin, const osg_zpulse *zp, void *e, void *b)
{
    if (!(dim == 2 || dim == 3) || order < 1 || order > 4 || !nx || !gcl || !gcu || !dx ||
        !xmin || !zp || !e || !b || (precision != 32 && precision != 64))
        return OSG_ERR_ARG;
    if (!(zp->lon_duration > 0) || !(zp->per_w0 > 0) || !(zp->omega0 > 0))
        return OSG_ERR_ARG;
    if (precision == 32)
        launch<float>(dim, order, nx, gcl, gcu, dx, xmin, *zp, (float *)e, (float *)b);
    else
        launch<double>(dim, order, nx, gcl, gcu, dx, xmin, *zp, (double *)e, (double *)b);
    return OSG_OK;
}
