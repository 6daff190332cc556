"""ORACLE — test infrastructure only: the CPU restatement of the reference
operators (oracle.cpp) used as the checker and the timed CPU baseline."""
