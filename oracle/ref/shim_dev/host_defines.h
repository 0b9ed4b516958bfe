/* host_defines.h stand-in for the device build: nvcc already provides the qualifiers */
