/* Force-included when compiling the reference sources out of tree.
 * Newer glibc defines CHAR_WIDTH in <limits.h>; the fmt copy bundled with the
 * reference's spdlog (src/thirdparty/spdlog/fmt/bundled/format.h:2198) uses the
 * same name for an enum member.  Pull <climits> in first, then drop the macro. */
#include <climits>
#undef CHAR_WIDTH
