/* The C-ABI from plain C11 (what a cgo / JNI / ctypes binding sees):
 * include/ttg.h compiles with -pedantic, and the entry points answer the
 * argument checks that come before any device work. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "ttg.h"

static int failed = 0;
#define CHECK(cond, msg)              \
  do                                  \
  {                                   \
    if (!(cond))                      \
    {                                 \
      printf("FAIL: %s\n", msg);      \
      ++failed;                       \
    }                                 \
  } while (0)

int main(void)
{
  CHECK(strcmp(ttg_status_string(TTG_OK), "ok") == 0, "status string");

  /* a two-site TT with consistent ranks, in the reference's layout */
  int32_t ranks[3] = {1, 2, 1}, rows[2] = {2, 3};
  int64_t offsets[3] = {0, 4, 10};
  double data[10] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10};
  ttg_tensor t;
  memset(&t, 0, sizeof(t));
  t.d = 2;
  t.ranks = ranks;
  t.rows = rows;
  t.offsets = offsets;
  t.data = data;

  ttg_tensor out;
  memset(&out, 0, sizeof(out));
  CHECK(ttg_round(&t, NULL, &out, NULL) == TTG_ERR_ARG, "round: null options");
  ttg_round_options o;
  memset(&o, 0, sizeof(o));
  o.eps = -1.0;
  CHECK(ttg_round(&t, &o, &out, NULL) == TTG_ERR_ARG, "round: negative eps");
  o.eps = 1e-8;
  o.method = TTG_METHOD_SVD_STREAMING;
  CHECK(ttg_round(&t, &o, &out, NULL) == TTG_ERR_METHOD, "round: streaming method");

  CHECK(ttg_soft_threshold(&t, NAN, &out) == TTG_ERR_ARG, "soft_threshold: NaN tau");
  CHECK(ttg_soft_threshold(&t, 0.0, &out) == TTG_OK, "soft_threshold: tau = 0 copies");
  CHECK(out.owned && out.d == 2 && out.data[9] == 10.0, "soft_threshold copy content");
  ttg_free(&out);
  CHECK(out.data == NULL, "ttg_free clears");

  ranks[1] = 3; /* offsets no longer match the core sizes */
  double v = -1.0;
  CHECK(ttg_inner(&t, &t, &v) == TTG_ERR_SHAPE, "inner: ragged input");
  ttg_tensor empty;
  memset(&empty, 0, sizeof(empty));
  CHECK(ttg_frob_norm_apply(&empty, &empty, &v) == TTG_OK && v == 0.0, "frob_norm_apply d=0");

  if (failed == 0)
    printf("test_c_abi: OK\n");
  return failed;
}
