/* Minimal build configuration for compiling the reference's portable C
 * primitives as a CPU checker: 8-bit, no x86 SIMD, POSIX threads.  Written
 * for this project (the reference's own configure script is not used). */
#define ARCH_X86            0
#define ARCH_X86_64         0
#define ARCH_PPC            0
#define ARCH_ARM            0
#define SYS_LINUX           1
#define SYS_WINDOWS         0
#define SYS_MACOSX          0
#define HAVE_MMX            0
#define HAVE_THREAD         1
#define HAVE_POSIXTHREAD    1
#define HAVE_WIN32THREAD    0
#define HAVE_BEOSTHREAD     0
#define HAVE_STDINT_H       1
#define HAVE_LOG2F          1
#define HAVE_MALLOC_H       1
#define HAVE_X86_INLINE_ASM 0
#define BIT_DEPTH           8
