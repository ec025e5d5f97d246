/* nbgb_status.h -- status codes of the GB300 n-body library (C ABI). */
#ifndef NBGB_STATUS_H
#define NBGB_STATUS_H

/* Return codes of the int-returning entry points (0 = success). */
#define NBGB_OK 0
#define NBGB_ERR_INVALID_ARGUMENT -1 /* null pointer, bad size, bad mode     */
#define NBGB_ERR_WORKSPACE -2        /* workspace missing or too small       */
#define NBGB_ERR_CUDA -3             /* a CUDA runtime call failed           */
#define NBGB_ERR_DEVICE -4           /* a kernel reported a device status    */
#define NBGB_ERR_UNSUPPORTED -5      /* device is not sm_103 / not supported */
#define NBGB_ERR_NO_MEMORY -6        /* allocation (or memory budget) failed */
#define NBGB_ERR_TOO_LARGE -7        /* size exceeds a documented maximum    */

/* Bits of the device status word (nbgb_last_status). */
#define NBGB_STATUS_WAIT_TIMEOUT 0x1u /* a bounded mbarrier wait ran out     */
#define NBGB_STATUS_QUEUE_TIMEOUT 0x2u /* a bounded work-queue wait ran out  */
#define NBGB_STATUS_BAD_PLAN 0x4u     /* kernel saw an inconsistent plan     */
#define NBGB_STATUS_NEGATIVE_MASS 0x8u /* a log-domain plan met a mass < 0   */

#endif
