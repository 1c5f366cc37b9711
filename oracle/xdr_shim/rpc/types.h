/*
 * Minimal stand-in for <rpc/types.h>, written for this project so that the
 * reference skid sources compile on hosts without SunRPC/tirpc.  Only the
 * names the reference uses are declared.
 */
#ifndef SKID_SHIM_RPC_TYPES_H
#define SKID_SHIM_RPC_TYPES_H

typedef int bool_t;

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif

#endif
