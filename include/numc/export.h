/* Symbol visibility for the numc-compatible GB300 library.
 * Same macro name and meaning as numc's include/numc/export.h:1-24. */
#ifndef NUMC_EXPORT_H
#define NUMC_EXPORT_H

#if defined(NUMC_STATIC_DEFINE)
#define NUMC_API
#elif !defined(NUMC_API)
#if defined(__GNUC__) && __GNUC__ >= 4
#define NUMC_API __attribute__((visibility("default")))
#else
#define NUMC_API
#endif
#endif

#endif /* NUMC_EXPORT_H */
