/* Exported configuration stand-in (8-bit, 4:2:0) for the CPU checker build. */
#define XAVS2_BIT_DEPTH     8
#define XAVS2_GPL           1
#define XAVS2_INTERLACED    0
#define XAVS2_CHROMA_FORMAT XAVS2_CSP_I420
