// Error text shared by the library's translation units.
#pragma once

namespace drmlt {

// Records msg as this thread's drmlt_last_error() text and returns code.
int set_error(int code, const char *msg);

}  // namespace drmlt
