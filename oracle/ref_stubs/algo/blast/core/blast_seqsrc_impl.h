/* Stub (see blast_extend.h): included by gpu_cpu_common.h, nothing used. */
#pragma once
