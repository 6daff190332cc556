"""ORACLE — test infrastructure only: the CPU restatement of the reference
operators (oracle.cpp), against which the parity tests compare the CUDA path, and
the timed CPU baseline."""
