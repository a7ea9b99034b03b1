/* aarch64 stand-in for the one x86 intrinsic the reference's scalar set
 * intersection uses (a prefetch hint). */
#pragma once
#define _MM_HINT_T0 3
#define _mm_prefetch(p, hint) __builtin_prefetch((const void *)(p))
