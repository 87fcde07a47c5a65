/* Minimal build configuration used when the reference's hot-path sources are
 * compiled directly (without their CMake project) into the headless oracle
 * driver under oracle/_ref/.  Only the switches that the compiled sources test
 * are defined; optional libraries (LASzip, Plytapus, Mitobrevno) are off.
 */
#ifndef CONFIG_H
#define CONFIG_H
#define HAVE_TIME_H
#define HAVE_SYS_TIME_H
#define HAVE_SYS_RESOURCE_H
#define HAVE_SYS_SYSINFO_H
#define HAVE_PROC_MEMINFO
#define SYSTEM_NAME Linux
#define SYSTEM_VERSION 0
#define VERSION "oracle"
#define COPY_YEAR 2023
#define SHARE_DIR "/nonexistent"
#endif
