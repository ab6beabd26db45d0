/* Type names only: the single-rank oracle build never partitions. */
#ifndef REFSHIM_PARMETIS_H
#define REFSHIM_PARMETIS_H
#include <stdint.h>
typedef int32_t idx_t;
typedef float real_t;
#endif
