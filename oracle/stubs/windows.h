/* Test-infrastructure stub (oracle build only): the reference's process.cxx
 * lowers its own priority through Win32; on Linux that is a no-op. */
#pragma once
typedef unsigned long DWORD;
#define NORMAL_PRIORITY_CLASS 0
#define IDLE_PRIORITY_CLASS 0
static inline void *GetCurrentProcess(void) { return 0; }
static inline int SetPriorityClass(void *, int) { return 1; }
static inline DWORD GetLastError(void) { return 0; }
