/* Empty configuration header standing in for the autotools-generated one.
 * Only the oracle's reference build (oracle/ref/Makefile) uses it. */
#ifndef ORACLE_REF_SUZERAIN_CONFIG_H
#define ORACLE_REF_SUZERAIN_CONFIG_H
#endif
