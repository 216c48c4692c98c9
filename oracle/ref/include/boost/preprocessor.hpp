/* Empty stand-in: suzerain/common.h includes Boost.Preprocessor, which the
 * translation units of the oracle's reference build never expand. */
