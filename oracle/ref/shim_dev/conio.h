/* conio.h stand-in (Windows console header, unused by the kernels) */
