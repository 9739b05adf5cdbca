/*
 * pcg_loader.c -- dlopen front end of the xJPCG C API.
 *
 * Drop-in for the reference's libXilinxPcg_loader.a (pcg/sw/src/pcg_loader.c,
 * built by pcg/sw/Makefile:112-177): an application links this archive (with
 * -ldl) instead of libXilinxPcg.so, and every xJPCG_* call resolves its
 * target in "libXilinxPcgStatic.so" on first use.  The library is looked up
 * on the normal dynamic-linker path (LD_LIBRARY_PATH); in this repository the
 * name is a symlink to hpc_gb300/libXilinxPcg.so.
 *
 * Behaviour kept from the reference:
 *   - an already loaded copy of the library is reused (RTLD_NOLOAD first),
 *     otherwise it is opened RTLD_LAZY | RTLD_GLOBAL;
 *   - a failed open or a missing symbol makes the call return
 *     XJPCG_STATUS_DYNAMIC_LOADING_ERROR and stores one process-wide message
 *     (pcg.h:232-234: not thread safe to read);
 *   - xJPCG_peekAtLastStatus and xJPCG_getLastMessage report a stored loading
 *     error without touching the library, so they work with a null handle;
 *   - xJPCG_getErrorString answers XJPCG_STATUS_DYNAMIC_LOADING_ERROR itself;
 *   - a successful resolution clears the stored error.
 *
 * The library handle is opened once and kept; each forwarding function keeps
 * the address it resolved, so a call after the first costs one atomic load
 * and adds no dlopen reference.  A failed open or lookup is retried on the
 * next call.  Writes of the process-wide message are serialised by a spin
 * lock (GCC atomics, no pthread dependency); as in the reference, a pointer
 * returned by xJPCG_getLastMessage may be overwritten by another thread's
 * later failure.
 *
 * Compile with XILINX_PCG_INLINE_IMPL (and include pcg.h with
 * XILINX_PCG_INLINE) to use this file as a header-only loader from C++.
 */
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>

#include "pcg.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifdef XILINX_PCG_INLINE_IMPL
#define XJL_DEF inline
#else
#define XJL_DEF
#endif

#define XJL_LIBRARY "libXilinxPcgStatic.so"
#define XJL_MSG_CAP 4096

/* Process-wide loading error: empty string = none. */
static char xjl_message[XJL_MSG_CAP];
static int xjl_message_lock;   /* spin lock over writes of xjl_message */
static void* xjl_library;      /* the opened library, once opened */

static const char* xjl_stored_error(void) {
    return __atomic_load_n(&xjl_message[0], __ATOMIC_ACQUIRE) ? xjl_message : NULL;
}

static void xjl_lock(void) {
    while (__atomic_test_and_set(&xjl_message_lock, __ATOMIC_ACQUIRE)) {
    }
}

static void xjl_unlock(void) { __atomic_clear(&xjl_message_lock, __ATOMIC_RELEASE); }

static void xjl_store_error(const char* what, const char* name, const char* why) {
    xjl_lock();
    snprintf(xjl_message, XJL_MSG_CAP,
             "ERROR: dynamic loading of the xJPCG library failed: %s %s (%s). The directory holding %s must be on "
             "LD_LIBRARY_PATH, and the library must be this interface's version.\n",
             what, name, why ? why : "unknown reason", XJL_LIBRARY);
    xjl_unlock();
}

static void xjl_clear_error(void) {
    if (__atomic_load_n(&xjl_message[0], __ATOMIC_ACQUIRE) == '\0') return;
    xjl_lock();
    __atomic_store_n(&xjl_message[0], '\0', __ATOMIC_RELEASE);
    xjl_unlock();
}

/* The library handle: opened on first use and kept for the process. */
static void* xjl_open(void) {
    void* lib = __atomic_load_n(&xjl_library, __ATOMIC_ACQUIRE);
    if (lib != NULL) return lib;
    lib = dlopen(XJL_LIBRARY, RTLD_LAZY | RTLD_NOLOAD);
    if (lib == NULL) lib = dlopen(XJL_LIBRARY, RTLD_LAZY | RTLD_GLOBAL);
    if (lib == NULL) {
        xjl_store_error("cannot open", XJL_LIBRARY, dlerror());
        return NULL;
    }
    void* expected = NULL;
    if (!__atomic_compare_exchange_n(&xjl_library, &expected, lib, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE)) {
        dlclose(lib); /* another thread stored its handle first: drop this reference */
        lib = expected;
    }
    return lib;
}

/* Address of `name` in the library, resolved once into *cache, or NULL with
 * the error stored. */
static void* xjl_symbol(const char* name, void** cache) {
    void* fn = __atomic_load_n(cache, __ATOMIC_ACQUIRE);
    if (fn != NULL) {
        xjl_clear_error();
        return fn;
    }
    void* lib = xjl_open();
    if (lib == NULL) return NULL;
    (void)dlerror();
    fn = dlsym(lib, name);
    const char* err = dlerror();
    if (err != NULL || fn == NULL) {
        xjl_store_error("cannot find symbol", name, err);
        return NULL;
    }
    __atomic_store_n(cache, fn, __ATOMIC_RELEASE);
    xjl_clear_error();
    return fn;
}

/* One resolved address per forwarded function. */
#define XJL_RESOLVE(name) (xjl_symbol(#name, &xjl_cache_##name))
static void* xjl_cache_xJPCG_createHandle;
static void* xjl_cache_xJPCG_destroyHandle;
static void* xjl_cache_xJPCG_getMetrics;
static void* xjl_cache_xJPCG_peekAtLastStatus;
static void* xjl_cache_xJPCG_getLastMessage;
static void* xjl_cache_xJPCG_getErrorString;
static void* xjl_cache_xJPCG_cscSymSolver;
static void* xjl_cache_xJPCG_cooSolver;

XJL_DEF
XJPCG_Status_t xJPCG_createHandle(XJPCG_Handle_t** handle, const char* xclbinPath) {
    typedef XJPCG_Status_t (*Fn)(XJPCG_Handle_t**, const char*);
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_createHandle);
    return fn ? fn(handle, xclbinPath) : XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
}

XJL_DEF
XJPCG_Status_t xJPCG_destroyHandle(XJPCG_Handle_t* handle) {
    typedef XJPCG_Status_t (*Fn)(XJPCG_Handle_t*);
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_destroyHandle);
    return fn ? fn(handle) : XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
}

XJL_DEF
XJPCG_Status_t xJPCG_getMetrics(const XJPCG_Handle_t* handle, XJPCG_Metric_t* metric) {
    typedef XJPCG_Status_t (*Fn)(const XJPCG_Handle_t*, XJPCG_Metric_t*);
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_getMetrics);
    return fn ? fn(handle, metric) : XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
}

XJL_DEF
XJPCG_Status_t xJPCG_peekAtLastStatus(const XJPCG_Handle_t* handle) {
    typedef XJPCG_Status_t (*Fn)(const XJPCG_Handle_t*);
    if (xjl_stored_error() != NULL) return XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_peekAtLastStatus);
    return fn ? fn(handle) : XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
}

XJL_DEF
const char* xJPCG_getLastMessage(const XJPCG_Handle_t* handle) {
    typedef const char* (*Fn)(const XJPCG_Handle_t*);
    const char* stored = xjl_stored_error();
    if (stored != NULL) return stored;
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_getLastMessage);
    if (fn != NULL) return fn(handle);
    return xjl_stored_error();
}

XJL_DEF
const char* xJPCG_getErrorString(const XJPCG_Status_t code) {
    typedef const char* (*Fn)(const XJPCG_Status_t);
    if (code == XJPCG_STATUS_DYNAMIC_LOADING_ERROR) return "Dynamic loading error";
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_getErrorString);
    return fn ? fn(code) : "ERROR: the error string is unavailable: the xJPCG library could not be loaded.";
}

XJL_DEF
XJPCG_Status_t xJPCG_cscSymSolver(XJPCG_Handle_t* handle, const int64_t p_n, const int64_t p_nnz,
                                  const int64_t* p_rowIdx, const int64_t* p_colPtr, const double* p_data,
                                  const double* matJ, const double* b, const double* x, const int64_t p_maxIter,
                                  const double p_tol, int64_t* p_iter, double* p_res, const XJPCG_Mode_t mode) {
    typedef XJPCG_Status_t (*Fn)(XJPCG_Handle_t*, const int64_t, const int64_t, const int64_t*, const int64_t*,
                                 const double*, const double*, const double*, const double*, const int64_t,
                                 const double, int64_t*, double*, const XJPCG_Mode_t);
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_cscSymSolver);
    if (fn == NULL) return XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
    return fn(handle, p_n, p_nnz, p_rowIdx, p_colPtr, p_data, matJ, b, x, p_maxIter, p_tol, p_iter, p_res, mode);
}

XJL_DEF
XJPCG_Status_t xJPCG_cooSolver(XJPCG_Handle_t* handle, const uint32_t p_n, const uint32_t p_nnz,
                               const uint32_t* p_rowIdx, const uint32_t* p_colIdx, const double* p_data,
                               const double* matJ, const double* b, const double* x, const uint32_t p_maxIter,
                               const double p_tol, uint32_t* p_iter, double* p_res, const XJPCG_Mode_t mode) {
    typedef XJPCG_Status_t (*Fn)(XJPCG_Handle_t*, const uint32_t, const uint32_t, const uint32_t*,
                                 const uint32_t*, const double*, const double*, const double*, const double*,
                                 const uint32_t, const double, uint32_t*, double*, const XJPCG_Mode_t);
    Fn fn = (Fn)XJL_RESOLVE(xJPCG_cooSolver);
    if (fn == NULL) return XJPCG_STATUS_DYNAMIC_LOADING_ERROR;
    return fn(handle, p_n, p_nnz, p_rowIdx, p_colIdx, p_data, matJ, b, x, p_maxIter, p_tol, p_iter, p_res, mode);
}

#ifdef __cplusplus
}
#endif
