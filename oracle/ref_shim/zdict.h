/* Declaration-only stand-in for <zdict.h> (see mpi.h in this directory). */
#pragma once
