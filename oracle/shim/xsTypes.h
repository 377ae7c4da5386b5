/* xsTypes.h -- stand-in for the one XSPEC typedef the reference uses
 * (XspecSpectrum.h:22). */
#ifndef RELX_ORACLE_XSTYPES_H
#define RELX_ORACLE_XSTYPES_H
#include <valarray>
typedef std::valarray<double> RealArray;
#endif
