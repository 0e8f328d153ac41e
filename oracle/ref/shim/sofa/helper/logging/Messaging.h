// Stand-in for the reference's logging header: the math code only streams
// warnings, so every msg_* macro becomes a sink that discards its input.
#pragma once
#include <ostream>
namespace oracle_ref_shim {
struct NullStream {
    template <class T> NullStream& operator<<(const T&) { return *this; }
    NullStream& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
}
#define msg_warning(...) oracle_ref_shim::NullStream()
#define msg_error(...) oracle_ref_shim::NullStream()
#define msg_info(...) oracle_ref_shim::NullStream()
#define dmsg_warning(...) oracle_ref_shim::NullStream()
#define dmsg_error(...) oracle_ref_shim::NullStream()
#define dmsg_info(...) oracle_ref_shim::NullStream()
#define msgendl "\n"
