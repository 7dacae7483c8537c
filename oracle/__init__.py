"""CPU oracle for the occluder rasteriser (test infrastructure only).

Only the tests, the smoke check and the CPU-baseline leg of the benchmark
import this package, and only to check results or as the timed CPU baseline.
"""
