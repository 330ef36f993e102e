/* Empty stand-in: DAKC's counting sources include <immintrin.h> but only use
 * it inside `#if 0` blocks, and AArch64 hosts have no such header. */
