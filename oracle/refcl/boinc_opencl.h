/*
 * boinc_opencl.h -- stand-in for the BOINC OpenCL device query, for the
 * standalone build of the reference program (see boinc_api.h).  Without a
 * client there is no init_data.xml to name a device, so the query fails and
 * the program takes platform 0, device 0, as it does when run by hand.
 */
#ifndef PFC_REFCL_BOINC_OPENCL_H
#define PFC_REFCL_BOINC_OPENCL_H

#ifndef CL_TARGET_OPENCL_VERSION
#define CL_TARGET_OPENCL_VERSION 110
#endif
#include "cl.h"

inline int boinc_get_opencl_ids(int, char **, int, cl_device_id *, cl_platform_id *) { return 1; }

#endif
