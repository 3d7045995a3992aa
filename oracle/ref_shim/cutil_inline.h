/* Empty stand-in: the reference helper files include this header but use
 * nothing from it (oracle build only). */
#ifndef FG_SHIM_CUTIL_INLINE_H
#define FG_SHIM_CUTIL_INLINE_H
#endif
