/*
 * Compatibility header with the reference's name (src/common.h): the
 * standard headers it pulls in, its error and logging macros and its small
 * inline helpers, so that callers written against libfmftsaxs compile
 * unchanged against fmftsaxs-gb300.
 */
#ifndef FMFTSAXS_GB300_COMPAT_COMMON_H
#define FMFTSAXS_GB300_COMPAT_COMMON_H

#include <assert.h>
#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "define.h"

/* print where the error happened and end the process */
#define ERROR_MSG(msg)                                                                                  \
	{                                                                                                   \
		fprintf(stderr, "[Error] %s, function %s, line %i: %s\n", __FILE__, __func__, __LINE__, msg); \
		exit(EXIT_FAILURE);                                                                             \
	}

#define CHECK_PTR(ptr)                   \
	{                                    \
		if ((ptr) == NULL) {             \
			ERROR_MSG("Null pointer");   \
		}                                \
	}

/* progress messages only in verbose builds */
#ifdef _SXS_VERBOSE_
#define SXS_PRINTF(...) printf(__VA_ARGS__)
#else
#define SXS_PRINTF(...)
#endif

/* index of A_lm in the coefficient arrays */
static inline int lm_index(int l, int m) { return l * (l + 1) + m; }

static inline void sxs_myfree(void *ptr)
{
	if (ptr != NULL) free(ptr);
}

static inline FILE *sxs_myfopen(char *path, char *mode)
{
	FILE *f = fopen(path, mode);
	if (f == NULL) {
		fprintf(stderr, "Unable to open %s\n", path);
		exit(EXIT_FAILURE);
	}
	return f;
}

#endif
