/*
 * cl_dispatch.c -- the OpenCL 1.1 entry points that the reference program
 * (mfl0p/PFCSieve: main.cpp, cl_sieve.cpp, simpleCL.c) calls, routed to a
 * vendor OpenCL implementation without a system ICD loader.
 *
 * TEST INFRASTRUCTURE: linked only into oracle/_ref/pfcsieve_ref, the
 * reference's own OpenCL program built from its sources so that bench.py can
 * time it on the same GPU.  Nothing in pfcsieve_gb300 uses OpenCL.
 *
 * Why it exists: the GPU machines carry NVIDIA's vendor library
 * (libnvidia-opencl.so.1) but no libOpenCL.so and no /etc/OpenCL/vendors
 * registration.  A vendor library of the Khronos installable-client-driver
 * (ICD) scheme exports clGetExtensionFunctionAddress, through which its
 * clIcdGetPlatformIDsKHR is found; every object it returns (platform, device,
 * context, queue, memory, program, kernel, event) starts with a pointer to
 * the vendor's table of entry points, in the order the Khronos ICD dispatch
 * table fixes for OpenCL 1.0 (the index constants below).  Each function here
 * reads that table from its first object argument and calls the vendor.
 *
 * The vendor library is PFC_OPENCL_VENDOR_LIB if set, else
 * libnvidia-opencl.so.1.  oracle/_ref/refcl_check (refcl_check.c) queries every
 * object kind through this table before the reference program runs, so a
 * wrong index shows up as a failed query and not as a wrong call.
 */
#define CL_TARGET_OPENCL_VERSION 110
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#include "cl.h"

/* positions in the vendor's dispatch table (OpenCL 1.0 section) */
enum {
    IX_GetPlatformInfo = 1,
    IX_GetDeviceIDs = 2,
    IX_GetDeviceInfo = 3,
    IX_CreateContext = 4,
    IX_ReleaseContext = 7,
    IX_GetContextInfo = 8,
    IX_CreateCommandQueue = 9,
    IX_ReleaseCommandQueue = 11,
    IX_GetCommandQueueInfo = 12,
    IX_CreateBuffer = 14,
    IX_ReleaseMemObject = 18,
    IX_GetMemObjectInfo = 20,
    IX_CreateProgramWithSource = 26,
    IX_ReleaseProgram = 29,
    IX_BuildProgram = 30,
    IX_GetProgramInfo = 32,
    IX_GetProgramBuildInfo = 33,
    IX_CreateKernel = 34,
    IX_ReleaseKernel = 37,
    IX_SetKernelArg = 38,
    IX_GetKernelInfo = 39,
    IX_GetKernelWorkGroupInfo = 40,
    IX_WaitForEvents = 41,
    IX_GetEventInfo = 42,
    IX_ReleaseEvent = 44,
    IX_GetEventProfilingInfo = 45,
    IX_Flush = 46,
    IX_Finish = 47,
    IX_EnqueueReadBuffer = 48,
    IX_EnqueueWriteBuffer = 49,
    IX_EnqueueNDRangeKernel = 59,
    IX_EnqueueMarker = 62,
};

/* the vendor's table of an ICD object */
static void *const *table_of(const void *obj) { return *(void *const *const *)obj; }

#define VENDOR_FN(obj, ix, type) ((type)table_of(obj)[ix])

typedef cl_int (*icd_platforms_fn)(cl_uint, cl_platform_id *, cl_uint *);
typedef void *(*ext_addr_fn)(const char *);

static icd_platforms_fn g_platforms = NULL;

static int load_vendor(void) {
    if (g_platforms) return 1;
    const char *name = getenv("PFC_OPENCL_VENDOR_LIB");
    void *h = dlopen(name && *name ? name : "libnvidia-opencl.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        fprintf(stderr, "cl_dispatch: no OpenCL vendor library (%s)\n", dlerror());
        return 0;
    }
    ext_addr_fn ext = (ext_addr_fn)dlsym(h, "clGetExtensionFunctionAddress");
    if (ext) g_platforms = (icd_platforms_fn)ext("clIcdGetPlatformIDsKHR");
    if (!g_platforms) g_platforms = (icd_platforms_fn)dlsym(h, "clIcdGetPlatformIDsKHR");
    if (!g_platforms) fprintf(stderr, "cl_dispatch: vendor library has no clIcdGetPlatformIDsKHR\n");
    return g_platforms != NULL;
}

CL_API_ENTRY cl_int CL_API_CALL clGetPlatformIDs(cl_uint num_entries, cl_platform_id *platforms,
                                                 cl_uint *num_platforms) {
    if (!load_vendor()) return -1001;  /* CL_PLATFORM_NOT_FOUND_KHR */
    return g_platforms(num_entries, platforms, num_platforms);
}

CL_API_ENTRY cl_int CL_API_CALL clGetPlatformInfo(cl_platform_id pl, cl_platform_info what, size_t size,
                                                  void *value, size_t *size_ret) {
    if (!pl) return CL_INVALID_PLATFORM;
    return VENDOR_FN(pl, IX_GetPlatformInfo, cl_int (*)(cl_platform_id, cl_platform_info, size_t, void *,
                                                        size_t *))(pl, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clGetDeviceIDs(cl_platform_id pl, cl_device_type type, cl_uint num_entries,
                                               cl_device_id *devices, cl_uint *num_devices) {
    if (!pl) return CL_INVALID_PLATFORM;
    return VENDOR_FN(pl, IX_GetDeviceIDs, cl_int (*)(cl_platform_id, cl_device_type, cl_uint, cl_device_id *,
                                                     cl_uint *))(pl, type, num_entries, devices, num_devices);
}

CL_API_ENTRY cl_int CL_API_CALL clGetDeviceInfo(cl_device_id dev, cl_device_info what, size_t size, void *value,
                                                size_t *size_ret) {
    if (!dev) return CL_INVALID_DEVICE;
    return VENDOR_FN(dev, IX_GetDeviceInfo, cl_int (*)(cl_device_id, cl_device_info, size_t, void *,
                                                       size_t *))(dev, what, size, value, size_ret);
}

CL_API_ENTRY cl_context CL_API_CALL clCreateContext(const cl_context_properties *props, cl_uint num_devices,
                                                    const cl_device_id *devices,
                                                    void(CL_CALLBACK *notify)(const char *, const void *,
                                                                              size_t, void *),
                                                    void *user_data, cl_int *err) {
    if (!num_devices || !devices || !devices[0]) {
        if (err) *err = CL_INVALID_VALUE;
        return NULL;
    }
    typedef cl_context (*fn)(const cl_context_properties *, cl_uint, const cl_device_id *,
                             void(CL_CALLBACK *)(const char *, const void *, size_t, void *), void *, cl_int *);
    return VENDOR_FN(devices[0], IX_CreateContext, fn)(props, num_devices, devices, notify, user_data, err);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseContext(cl_context ctx) {
    if (!ctx) return CL_INVALID_CONTEXT;
    return VENDOR_FN(ctx, IX_ReleaseContext, cl_int (*)(cl_context))(ctx);
}

CL_API_ENTRY cl_int CL_API_CALL clGetContextInfo(cl_context ctx, cl_context_info what, size_t size, void *value,
                                                 size_t *size_ret) {
    if (!ctx) return CL_INVALID_CONTEXT;
    return VENDOR_FN(ctx, IX_GetContextInfo, cl_int (*)(cl_context, cl_context_info, size_t, void *,
                                                        size_t *))(ctx, what, size, value, size_ret);
}

CL_API_ENTRY cl_command_queue CL_API_CALL clCreateCommandQueue(cl_context ctx, cl_device_id dev,
                                                               cl_command_queue_properties props, cl_int *err) {
    if (!ctx) {
        if (err) *err = CL_INVALID_CONTEXT;
        return NULL;
    }
    return VENDOR_FN(ctx, IX_CreateCommandQueue, cl_command_queue (*)(cl_context, cl_device_id,
                                                                      cl_command_queue_properties,
                                                                      cl_int *))(ctx, dev, props, err);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseCommandQueue(cl_command_queue q) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    return VENDOR_FN(q, IX_ReleaseCommandQueue, cl_int (*)(cl_command_queue))(q);
}

CL_API_ENTRY cl_int CL_API_CALL clGetCommandQueueInfo(cl_command_queue q, cl_command_queue_info what, size_t size,
                                                      void *value, size_t *size_ret) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    return VENDOR_FN(q, IX_GetCommandQueueInfo, cl_int (*)(cl_command_queue, cl_command_queue_info, size_t,
                                                           void *, size_t *))(q, what, size, value, size_ret);
}

CL_API_ENTRY cl_mem CL_API_CALL clCreateBuffer(cl_context ctx, cl_mem_flags flags, size_t size, void *host_ptr,
                                               cl_int *err) {
    if (!ctx) {
        if (err) *err = CL_INVALID_CONTEXT;
        return NULL;
    }
    return VENDOR_FN(ctx, IX_CreateBuffer, cl_mem (*)(cl_context, cl_mem_flags, size_t, void *,
                                                      cl_int *))(ctx, flags, size, host_ptr, err);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseMemObject(cl_mem m) {
    if (!m) return CL_INVALID_MEM_OBJECT;
    return VENDOR_FN(m, IX_ReleaseMemObject, cl_int (*)(cl_mem))(m);
}

CL_API_ENTRY cl_int CL_API_CALL clGetMemObjectInfo(cl_mem m, cl_mem_info what, size_t size, void *value,
                                                   size_t *size_ret) {
    if (!m) return CL_INVALID_MEM_OBJECT;
    return VENDOR_FN(m, IX_GetMemObjectInfo, cl_int (*)(cl_mem, cl_mem_info, size_t, void *,
                                                        size_t *))(m, what, size, value, size_ret);
}

CL_API_ENTRY cl_program CL_API_CALL clCreateProgramWithSource(cl_context ctx, cl_uint count, const char **strings,
                                                              const size_t *lengths, cl_int *err) {
    if (!ctx) {
        if (err) *err = CL_INVALID_CONTEXT;
        return NULL;
    }
    return VENDOR_FN(ctx, IX_CreateProgramWithSource, cl_program (*)(cl_context, cl_uint, const char **,
                                                                     const size_t *,
                                                                     cl_int *))(ctx, count, strings, lengths, err);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseProgram(cl_program p) {
    if (!p) return CL_INVALID_PROGRAM;
    return VENDOR_FN(p, IX_ReleaseProgram, cl_int (*)(cl_program))(p);
}

CL_API_ENTRY cl_int CL_API_CALL clBuildProgram(cl_program p, cl_uint num_devices, const cl_device_id *devices,
                                               const char *options,
                                               void(CL_CALLBACK *notify)(cl_program, void *), void *user_data) {
    if (!p) return CL_INVALID_PROGRAM;
    typedef cl_int (*fn)(cl_program, cl_uint, const cl_device_id *, const char *,
                         void(CL_CALLBACK *)(cl_program, void *), void *);
    return VENDOR_FN(p, IX_BuildProgram, fn)(p, num_devices, devices, options, notify, user_data);
}

CL_API_ENTRY cl_int CL_API_CALL clGetProgramInfo(cl_program p, cl_program_info what, size_t size, void *value,
                                                 size_t *size_ret) {
    if (!p) return CL_INVALID_PROGRAM;
    return VENDOR_FN(p, IX_GetProgramInfo, cl_int (*)(cl_program, cl_program_info, size_t, void *,
                                                      size_t *))(p, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clGetProgramBuildInfo(cl_program p, cl_device_id dev, cl_program_build_info what,
                                                      size_t size, void *value, size_t *size_ret) {
    if (!p) return CL_INVALID_PROGRAM;
    return VENDOR_FN(p, IX_GetProgramBuildInfo, cl_int (*)(cl_program, cl_device_id, cl_program_build_info,
                                                           size_t, void *,
                                                           size_t *))(p, dev, what, size, value, size_ret);
}

CL_API_ENTRY cl_kernel CL_API_CALL clCreateKernel(cl_program p, const char *name, cl_int *err) {
    if (!p) {
        if (err) *err = CL_INVALID_PROGRAM;
        return NULL;
    }
    return VENDOR_FN(p, IX_CreateKernel, cl_kernel (*)(cl_program, const char *, cl_int *))(p, name, err);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseKernel(cl_kernel k) {
    if (!k) return CL_INVALID_KERNEL;
    return VENDOR_FN(k, IX_ReleaseKernel, cl_int (*)(cl_kernel))(k);
}

CL_API_ENTRY cl_int CL_API_CALL clSetKernelArg(cl_kernel k, cl_uint index, size_t size, const void *value) {
    if (!k) return CL_INVALID_KERNEL;
    return VENDOR_FN(k, IX_SetKernelArg, cl_int (*)(cl_kernel, cl_uint, size_t, const void *))(k, index, size,
                                                                                                value);
}

CL_API_ENTRY cl_int CL_API_CALL clGetKernelInfo(cl_kernel k, cl_kernel_info what, size_t size, void *value,
                                                size_t *size_ret) {
    if (!k) return CL_INVALID_KERNEL;
    return VENDOR_FN(k, IX_GetKernelInfo, cl_int (*)(cl_kernel, cl_kernel_info, size_t, void *,
                                                     size_t *))(k, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clGetKernelWorkGroupInfo(cl_kernel k, cl_device_id dev,
                                                         cl_kernel_work_group_info what, size_t size, void *value,
                                                         size_t *size_ret) {
    if (!k) return CL_INVALID_KERNEL;
    return VENDOR_FN(k, IX_GetKernelWorkGroupInfo, cl_int (*)(cl_kernel, cl_device_id, cl_kernel_work_group_info,
                                                              size_t, void *,
                                                              size_t *))(k, dev, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clWaitForEvents(cl_uint num_events, const cl_event *events) {
    if (!num_events || !events || !events[0]) return CL_INVALID_VALUE;
    return VENDOR_FN(events[0], IX_WaitForEvents, cl_int (*)(cl_uint, const cl_event *))(num_events, events);
}

CL_API_ENTRY cl_int CL_API_CALL clGetEventInfo(cl_event ev, cl_event_info what, size_t size, void *value,
                                               size_t *size_ret) {
    if (!ev) return CL_INVALID_EVENT;
    return VENDOR_FN(ev, IX_GetEventInfo, cl_int (*)(cl_event, cl_event_info, size_t, void *,
                                                     size_t *))(ev, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clReleaseEvent(cl_event ev) {
    if (!ev) return CL_INVALID_EVENT;
    return VENDOR_FN(ev, IX_ReleaseEvent, cl_int (*)(cl_event))(ev);
}

CL_API_ENTRY cl_int CL_API_CALL clGetEventProfilingInfo(cl_event ev, cl_profiling_info what, size_t size,
                                                        void *value, size_t *size_ret) {
    if (!ev) return CL_INVALID_EVENT;
    return VENDOR_FN(ev, IX_GetEventProfilingInfo, cl_int (*)(cl_event, cl_profiling_info, size_t, void *,
                                                              size_t *))(ev, what, size, value, size_ret);
}

CL_API_ENTRY cl_int CL_API_CALL clFlush(cl_command_queue q) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    return VENDOR_FN(q, IX_Flush, cl_int (*)(cl_command_queue))(q);
}

CL_API_ENTRY cl_int CL_API_CALL clFinish(cl_command_queue q) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    return VENDOR_FN(q, IX_Finish, cl_int (*)(cl_command_queue))(q);
}

CL_API_ENTRY cl_int CL_API_CALL clEnqueueReadBuffer(cl_command_queue q, cl_mem buf, cl_bool blocking, size_t offset,
                                                    size_t size, void *ptr, cl_uint num_wait,
                                                    const cl_event *wait_list, cl_event *event) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    typedef cl_int (*fn)(cl_command_queue, cl_mem, cl_bool, size_t, size_t, void *, cl_uint, const cl_event *,
                         cl_event *);
    return VENDOR_FN(q, IX_EnqueueReadBuffer, fn)(q, buf, blocking, offset, size, ptr, num_wait, wait_list, event);
}

CL_API_ENTRY cl_int CL_API_CALL clEnqueueWriteBuffer(cl_command_queue q, cl_mem buf, cl_bool blocking,
                                                     size_t offset, size_t size, const void *ptr, cl_uint num_wait,
                                                     const cl_event *wait_list, cl_event *event) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    typedef cl_int (*fn)(cl_command_queue, cl_mem, cl_bool, size_t, size_t, const void *, cl_uint,
                         const cl_event *, cl_event *);
    return VENDOR_FN(q, IX_EnqueueWriteBuffer, fn)(q, buf, blocking, offset, size, ptr, num_wait, wait_list,
                                                   event);
}

CL_API_ENTRY cl_int CL_API_CALL clEnqueueNDRangeKernel(cl_command_queue q, cl_kernel k, cl_uint dims,
                                                       const size_t *offset, const size_t *global,
                                                       const size_t *local, cl_uint num_wait,
                                                       const cl_event *wait_list, cl_event *event) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    typedef cl_int (*fn)(cl_command_queue, cl_kernel, cl_uint, const size_t *, const size_t *, const size_t *,
                         cl_uint, const cl_event *, cl_event *);
    return VENDOR_FN(q, IX_EnqueueNDRangeKernel, fn)(q, k, dims, offset, global, local, num_wait, wait_list, event);
}

CL_API_ENTRY cl_int CL_API_CALL clEnqueueMarker(cl_command_queue q, cl_event *event) {
    if (!q) return CL_INVALID_COMMAND_QUEUE;
    return VENDOR_FN(q, IX_EnqueueMarker, cl_int (*)(cl_command_queue, cl_event *))(q, event);
}
