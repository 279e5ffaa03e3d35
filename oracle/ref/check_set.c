/* TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * The reference's heatbath-trajectory reader (src/hb_trajectory.c:156-160)
 * calls check_set(), which no source file of the reference defines, so its
 * -DHB_TRAJECTORY build does not link as shipped.  This definition lets the
 * reference binary su2_fundt build for the golden files: a key that was not
 * set ends the run with a message, as the other required config keys do. */
#include <stdio.h>
#include <stdlib.h>

void check_set(int set, const char* name) {
  if (!set) {
    printf("!!! Parameter %s not set in realtime_config! Exiting...\n", name);
    exit(-2);
  }
}
