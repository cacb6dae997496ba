/* Pre-included before any reference header when the reference is compiled
 * as the oracle. glibc's <limits.h> defines CHAR_WIDTH, which collides with
 * an enumerator of the same name in the vendored fmt library
 * (lib/utility/format.h). Pull <climits> in first, then drop the macro. */
#include <climits>
#undef CHAR_WIDTH
