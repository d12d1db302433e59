// Declarations only (TEST INFRASTRUCTURE ONLY): Core/Utils.hpp of the
// reference includes <Windows.h> for file-system helpers that the pinned
// kernels never call.  Nothing here is defined, linked or executed.
#pragma once
typedef void *HANDLE;
typedef unsigned long DWORD;
typedef struct {
    DWORD dwFileAttributes;
    char cFileName[260];
} WIN32_FIND_DATA;
#define CP_ACP 0
#define FILE_ATTRIBUTE_DIRECTORY 0x10
#define INVALID_HANDLE_VALUE ((HANDLE)(long)-1)
int SetCurrentDirectory(const char *);
int MultiByteToWideChar(unsigned, DWORD, const char *, int, wchar_t *, int);
HANDLE FindFirstFile(const char *, WIN32_FIND_DATA *);
int FindNextFile(HANDLE, WIN32_FIND_DATA *);
int FindClose(HANDLE);
