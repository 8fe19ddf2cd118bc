/*
 * jl_probe.c -- a thin shim over the reference's own jl gather-scatter
 * library (src/jl/gs.c, src/jl/gs_local.c and their support files), compiled
 * from the reference sources by oracle/Makefile into oracle/_ref/.
 *
 * TEST INFRASTRUCTURE ONLY: it exists so that the oracle's restatement of the
 * gather-scatter (oracle/nb_oracle.c) and, through it, the CUDA gather-scatter
 * maps can be pinned bit-exactly against the reference itself.
 *
 * The reference keeps struct gs_data private to gs.c (gs.c:1022-1027); the
 * view below repeats its leading members, which is what local_setup
 * (gs.c:1064-1069) fills: the unflagged map, the full map and the flagged
 * primaries.
 */
#include <float.h>
#include <limits.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "c99.h"
#include "name.h"
#include "fail.h"
#include "types.h"
#include "comm.h"
#include "mem.h"
#include "gs_defs.h"
#include "gs.h"

struct gs_data_view {
  struct comm comm;
  const uint *map_local[2];
  const uint *flagged_primaries;
};

static struct comm probe_comm;
static int probe_comm_ready = 0;

void *jlp_gs_setup(const long long *ids, int n) {
  if (!probe_comm_ready) {
    comm_init(&probe_comm, 0);
    probe_comm_ready = 1;
  }
  return gs_setup((const slong *)ids, (uint)n, &probe_comm, 0, gs_auto, 0);
}

/* dom 1..4 = double, float, int, long; op 1..4 = add, mul, min, max
 * (the Fortran numbering checked at gs.c:1172-1186) */
void jlp_gs_op(void *h, void *u, int dom, int op, int transpose) {
  gs(u, (gs_dom)(dom - 1), (gs_op)(op - 1), transpose != 0,
     (struct gs_data *)h, 0);
}

void jlp_gs_free(void *h) { gs_free((struct gs_data *)h); }

static const uint *view_map(void *h, int which) {
  const struct gs_data_view *v = (const struct gs_data_view *)h;
  return which == 2 ? v->flagged_primaries : v->map_local[which];
}

/* number of entries, counting every -1 terminator, of a map in the
 * format written by local_map (gs.c:330-357) */
int jlp_map_len(void *h, int which) {
  const uint *m = view_map(h, which);
  int n = 0;
  if (which == 2) {
    while (m[n] != (uint)-1) ++n;
    return n + 1;
  }
  for (;;) {
    if (m[n] == (uint)-1) return n + 1;
    ++n; /* primary */
    while (m[n] != (uint)-1) ++n;
    ++n; /* group terminator */
  }
}

void jlp_map_copy(void *h, int which, unsigned *out) {
  const uint *m = view_map(h, which);
  int n = jlp_map_len(h, which);
  for (int i = 0; i < n; ++i) out[i] = m[i];
}

void jlp_gs_unique(long long *ids, int n) {
  if (!probe_comm_ready) {
    comm_init(&probe_comm, 0);
    probe_comm_ready = 1;
  }
  gs_unique((slong *)ids, (uint)n, &probe_comm);
}
