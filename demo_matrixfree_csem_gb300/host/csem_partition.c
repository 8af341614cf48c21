/* Balanced split of independent systems over devices (include/csem_host.h). */
#include <math.h>
#include <stdlib.h>
#include "csem_host.h"

int csem_set_error(int code, const char *fmt, ...);

typedef struct {
  double w;
  int s;
} item_t;

static int by_work_desc(const void *a, const void *b)
{
  const item_t *x = (const item_t *)a, *y = (const item_t *)b;
  if (x->w > y->w) return -1;
  if (x->w < y->w) return 1;
  return x->s - y->s;
}

int csem_partition_systems(int nsys, const float *freq, const double *cost, double unknowns, int ndev, int *owner,
                           double *load)
{
  if (ndev < 1 || nsys < 0 || (nsys > 0 && !owner) || (nsys > 0 && !cost && !freq))
    return csem_set_error(CSEM_EINVAL, "csem_partition_systems: bad arguments");
  if (!cost && !(unknowns > 0)) return csem_set_error(CSEM_EINVAL, "csem_partition_systems: unknowns must be > 0");
  item_t *it = (item_t *)malloc(sizeof(item_t) * (size_t)(nsys > 0 ? nsys : 1));
  double *acc = (double *)calloc((size_t)ndev, sizeof(double));
  if (!it || !acc) {
    free(it);
    free(acc);
    return csem_set_error(CSEM_ENOMEM, "csem_partition_systems: out of memory");
  }
  for (int s = 0; s < nsys; s++) {
    const double w = cost ? cost[s] : (freq[s] > 0 ? unknowns * pow((double)freq[s], -2.0 / 3.0) : -1.0);
    if (!(w > 0) || !isfinite(w)) {
      free(it);
      free(acc);
      return csem_set_error(CSEM_EINVAL, "csem_partition_systems: system %d has no positive work", s);
    }
    it[s].w = w;
    it[s].s = s;
  }
  qsort(it, (size_t)nsys, sizeof(item_t), by_work_desc);
  for (int q = 0; q < nsys; q++) {
    int best = 0;
    for (int d = 1; d < ndev; d++)
      if (acc[d] < acc[best]) best = d;
    owner[it[q].s] = best;
    acc[best] += it[q].w;
  }
  if (load)
    for (int d = 0; d < ndev; d++) load[d] = acc[d];
  free(it);
  free(acc);
  return CSEM_OK;
}
