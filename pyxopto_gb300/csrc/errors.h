/* errors.h - the library-wide "last error" of the calling host thread. */
#pragma once
namespace mcgb_internal {
/* stores msg as mcgb_last_error() text and returns code */
int set_error(int code, const char *msg);
}
