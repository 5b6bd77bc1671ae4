/* Empty stand-in for the reference's viewer header: che.cpp includes it but
 * uses nothing from it on the geodesics path, and no graphics stack exists
 * where the oracle is built. */
#ifndef GP_ORACLE_STUB_VIEWER_H
#define GP_ORACLE_STUB_VIEWER_H
#endif
