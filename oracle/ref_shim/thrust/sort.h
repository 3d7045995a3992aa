/* Empty stand-in: the reference's kernel file includes thrust/sort.h for its
 * launchers, which the host build of the kernels leaves out (oracle build
 * only). */
#ifndef FG_SHIM_THRUST_SORT_H
#define FG_SHIM_THRUST_SORT_H
#endif
