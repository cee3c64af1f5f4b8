/* Minimal stand-in for <windows.h>: only the names the reference's headers
 * declare with (FBPG/mucat_file.h:160,189).  Used solely to compile the
 * reference's device code into oracle/_ref/. */
#pragma once
typedef unsigned long DWORD;
typedef void *LPVOID;
typedef void *HANDLE;
#define WINAPI
