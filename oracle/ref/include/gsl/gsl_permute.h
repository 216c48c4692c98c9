/* Empty stand-in: the reference's bsmbsm.h includes it, bsmbsm.c calls none of it. */
#ifndef ORACLE_REF_GSL_PERMUTE_H
#define ORACLE_REF_GSL_PERMUTE_H
#endif
