/* Stand-in for the reference's missing triangle_smooth.h: triangle_smooth.c
 * needs calloc/free only. */
#include <stdlib.h>
