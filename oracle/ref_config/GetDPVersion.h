/* Version header for the reference build made by oracle/build_ref.sh. */
#ifndef GETDP_VERSION_H
#define GETDP_VERSION_H
#define GETDP_MAJOR_VERSION 3
#define GETDP_MINOR_VERSION 5
#define GETDP_PATCH_VERSION 0
#define GETDP_EXTRA_VERSION ""
#define GETDP_VERSION "3.5.0"
#define GETDP_DATE "oracle-build"
#define GETDP_HOST "oracle"
#define GETDP_PACKAGER "oracle"
#define GETDP_OS "Linux64"
#define GETDP_SHORT_LICENSE "GNU General Public License"
#endif
