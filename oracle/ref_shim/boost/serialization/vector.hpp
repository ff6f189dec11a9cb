// Empty stand-in: the single-rank mpi stand-in never serialises objects.
#pragma once
