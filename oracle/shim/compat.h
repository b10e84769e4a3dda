/* Forced include for the oracle build of the reference: glibc removed
 * sys_errlist, which the vendored DT-Grid headers still name. */
#ifndef ESF_ORACLE_COMPAT_H
#define ESF_ORACLE_COMPAT_H
#ifdef __cplusplus
#include <cstring>
#include <cerrno>
#define sys_errlist esf_compat_sys_errlist()
namespace {
struct esf_errlist_proxy {
  const char* operator[](int e) const { return strerror(e); }
};
inline esf_errlist_proxy esf_compat_sys_errlist() { return esf_errlist_proxy(); }
}
#endif
#endif
