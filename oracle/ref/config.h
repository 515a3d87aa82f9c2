/*
 * config.h for compiling the reference KQED C library straight from its own
 * sources (test infrastructure only; see oracle/Makefile).
 *
 * The reference's autotools build generates this file; autotools is not used
 * here.  LIB_PATH is compile-time in the reference (configure.ac:24-27,
 * src/LIBFILES/io.c:10-12); here it expands to a function call so the table
 * directory can be chosen at run time through KQEDREF_PATH.
 */
#ifndef KQEDREF_CONFIG_H
#define KQEDREF_CONFIG_H

#if defined(__x86_64__) || defined(__i386__)
#define HAVE_IMMINTRIN_H 1
#endif
#define HAVE_OMP_H 1

const char *kqedref_lib_path(void);
#define LIB_PATH kqedref_lib_path()

#endif
