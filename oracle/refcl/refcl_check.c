/*
 * refcl_check.c -- check of cl_dispatch.c before the reference program runs.
 *
 * TEST INFRASTRUCTURE (see cl_dispatch.c).  Every table position that
 * cl_dispatch.c uses is exercised once, on objects of its kind, and each call
 * is followed by a query whose answer is known: the platform and device
 * names, the context's device, the queue's context and device, the buffer's
 * size, the program's device count, the kernel's name, the event's status and
 * timestamps, and the values a tiny kernel writes.  The kernel adds 1 to each
 * of 256 uints of a 1 KiB buffer with a global size of exactly 256, so it
 * stays inside its buffer whatever happens.  Exit status 0 when every answer
 * matches; the first mismatch is printed and the program exits 1.
 */
#define CL_TARGET_OPENCL_VERSION 110
#include <stdio.h>
#include <string.h>

#include "cl.h"

#define N 256

static int fail(const char *what, cl_int err) {
    printf("refcl_check: %s failed (%d)\n", what, (int)err);
    return 1;
}

int main(void) {
    cl_int err;
    cl_platform_id pl = NULL;
    cl_uint npl = 0;
    if ((err = clGetPlatformIDs(1, &pl, &npl)) != CL_SUCCESS || !pl) return fail("clGetPlatformIDs", err);
    char name[256] = {0};
    if ((err = clGetPlatformInfo(pl, CL_PLATFORM_NAME, sizeof name, name, NULL)) != CL_SUCCESS)
        return fail("clGetPlatformInfo", err);
    printf("platform: %s\n", name);

    cl_device_id dev = NULL;
    cl_uint ndev = 0;
    if ((err = clGetDeviceIDs(pl, CL_DEVICE_TYPE_GPU, 1, &dev, &ndev)) != CL_SUCCESS || !dev || ndev < 1)
        return fail("clGetDeviceIDs", err);
    char dname[256] = {0};
    cl_uint units = 0;
    if ((err = clGetDeviceInfo(dev, CL_DEVICE_NAME, sizeof dname, dname, NULL)) != CL_SUCCESS ||
        (err = clGetDeviceInfo(dev, CL_DEVICE_MAX_COMPUTE_UNITS, sizeof units, &units, NULL)) != CL_SUCCESS)
        return fail("clGetDeviceInfo", err);
    printf("device: %s, %u compute units\n", dname, units);
    if (!units) return fail("compute unit count", 0);

    cl_context_properties props[3] = {CL_CONTEXT_PLATFORM, (cl_context_properties)pl, 0};
    cl_context ctx = clCreateContext(props, 1, &dev, NULL, NULL, &err);
    if (!ctx || err != CL_SUCCESS) return fail("clCreateContext", err);
    cl_uint cnd = 0;
    cl_device_id cdev = NULL;
    if ((err = clGetContextInfo(ctx, CL_CONTEXT_NUM_DEVICES, sizeof cnd, &cnd, NULL)) != CL_SUCCESS || cnd != 1 ||
        (err = clGetContextInfo(ctx, CL_CONTEXT_DEVICES, sizeof cdev, &cdev, NULL)) != CL_SUCCESS || cdev != dev)
        return fail("clGetContextInfo", err);

    cl_command_queue q = clCreateCommandQueue(ctx, dev, CL_QUEUE_PROFILING_ENABLE, &err);
    if (!q || err != CL_SUCCESS) return fail("clCreateCommandQueue", err);
    cl_context qctx = NULL;
    cl_device_id qdev = NULL;
    if ((err = clGetCommandQueueInfo(q, CL_QUEUE_CONTEXT, sizeof qctx, &qctx, NULL)) != CL_SUCCESS || qctx != ctx ||
        (err = clGetCommandQueueInfo(q, CL_QUEUE_DEVICE, sizeof qdev, &qdev, NULL)) != CL_SUCCESS || qdev != dev)
        return fail("clGetCommandQueueInfo", err);

    cl_uint host[N];
    for (int i = 0; i < N; ++i) host[i] = 7u * (cl_uint)i;
    cl_mem buf = clCreateBuffer(ctx, CL_MEM_READ_WRITE, sizeof host, NULL, &err);
    if (!buf || err != CL_SUCCESS) return fail("clCreateBuffer", err);
    size_t msize = 0;
    if ((err = clGetMemObjectInfo(buf, CL_MEM_SIZE, sizeof msize, &msize, NULL)) != CL_SUCCESS ||
        msize != sizeof host)
        return fail("clGetMemObjectInfo", err);
    if ((err = clEnqueueWriteBuffer(q, buf, CL_TRUE, 0, sizeof host, host, 0, NULL, NULL)) != CL_SUCCESS)
        return fail("clEnqueueWriteBuffer", err);

    const char *src = "__kernel void add_one(__global uint *a, const uint n) {\n"
                      "  const uint i = get_global_id(0);\n"
                      "  if (i < n) a[i] += 1u;\n"
                      "}\n";
    cl_program prog = clCreateProgramWithSource(ctx, 1, &src, NULL, &err);
    if (!prog || err != CL_SUCCESS) return fail("clCreateProgramWithSource", err);
    if ((err = clBuildProgram(prog, 1, &dev, "", NULL, NULL)) != CL_SUCCESS) return fail("clBuildProgram", err);
    cl_build_status bst = CL_BUILD_NONE;
    cl_uint pnd = 0;
    if ((err = clGetProgramBuildInfo(prog, dev, CL_PROGRAM_BUILD_STATUS, sizeof bst, &bst, NULL)) != CL_SUCCESS ||
        bst != CL_BUILD_SUCCESS)
        return fail("clGetProgramBuildInfo", err);
    if ((err = clGetProgramInfo(prog, CL_PROGRAM_NUM_DEVICES, sizeof pnd, &pnd, NULL)) != CL_SUCCESS || pnd != 1)
        return fail("clGetProgramInfo", err);

    cl_kernel k = clCreateKernel(prog, "add_one", &err);
    if (!k || err != CL_SUCCESS) return fail("clCreateKernel", err);
    char kname[64] = {0};
    if ((err = clGetKernelInfo(k, CL_KERNEL_FUNCTION_NAME, sizeof kname, kname, NULL)) != CL_SUCCESS ||
        strcmp(kname, "add_one") != 0)
        return fail("clGetKernelInfo", err);
    size_t wg = 0;
    if ((err = clGetKernelWorkGroupInfo(k, dev, CL_KERNEL_WORK_GROUP_SIZE, sizeof wg, &wg, NULL)) != CL_SUCCESS ||
        wg < 1)
        return fail("clGetKernelWorkGroupInfo", err);
    const cl_uint n = N;
    if ((err = clSetKernelArg(k, 0, sizeof buf, &buf)) != CL_SUCCESS ||
        (err = clSetKernelArg(k, 1, sizeof n, &n)) != CL_SUCCESS)
        return fail("clSetKernelArg", err);

    const size_t global = N;
    cl_event ev = NULL;
    if ((err = clEnqueueNDRangeKernel(q, k, 1, NULL, &global, NULL, 0, NULL, &ev)) != CL_SUCCESS || !ev)
        return fail("clEnqueueNDRangeKernel", err);
    cl_event mark = NULL;
    if ((err = clEnqueueMarker(q, &mark)) != CL_SUCCESS || !mark) return fail("clEnqueueMarker", err);
    if ((err = clFlush(q)) != CL_SUCCESS) return fail("clFlush", err);
    if ((err = clWaitForEvents(1, &mark)) != CL_SUCCESS) return fail("clWaitForEvents", err);
    cl_int status = -1;
    if ((err = clGetEventInfo(ev, CL_EVENT_COMMAND_EXECUTION_STATUS, sizeof status, &status, NULL)) !=
            CL_SUCCESS ||
        status != CL_COMPLETE)
        return fail("clGetEventInfo", err);
    cl_ulong t0 = 0, t1 = 0;
    if ((err = clGetEventProfilingInfo(ev, CL_PROFILING_COMMAND_START, sizeof t0, &t0, NULL)) != CL_SUCCESS ||
        (err = clGetEventProfilingInfo(ev, CL_PROFILING_COMMAND_END, sizeof t1, &t1, NULL)) != CL_SUCCESS ||
        t1 < t0)
        return fail("clGetEventProfilingInfo", err);
    if ((err = clFinish(q)) != CL_SUCCESS) return fail("clFinish", err);

    cl_uint back[N];
    memset(back, 0, sizeof back);
    if ((err = clEnqueueReadBuffer(q, buf, CL_TRUE, 0, sizeof back, back, 0, NULL, NULL)) != CL_SUCCESS)
        return fail("clEnqueueReadBuffer", err);
    for (int i = 0; i < N; ++i)
        if (back[i] != host[i] + 1u) return fail("kernel result", i);

    if ((err = clReleaseEvent(ev)) != CL_SUCCESS || (err = clReleaseEvent(mark)) != CL_SUCCESS)
        return fail("clReleaseEvent", err);
    if ((err = clReleaseKernel(k)) != CL_SUCCESS) return fail("clReleaseKernel", err);
    if ((err = clReleaseProgram(prog)) != CL_SUCCESS) return fail("clReleaseProgram", err);
    if ((err = clReleaseMemObject(buf)) != CL_SUCCESS) return fail("clReleaseMemObject", err);
    if ((err = clReleaseCommandQueue(q)) != CL_SUCCESS) return fail("clReleaseCommandQueue", err);
    if ((err = clReleaseContext(ctx)) != CL_SUCCESS) return fail("clReleaseContext", err);
    printf("refcl_check: ok (kernel %.3f us)\n", (t1 - t0) / 1e3);
    return 0;
}
