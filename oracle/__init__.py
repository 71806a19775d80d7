"""ORACLE — test infrastructure only (the CPU restatement of the reference's hot path).

Imported by tests/, by the smoke check and by the CPU-baseline / reference legs of bench.py,
and nowhere else. The product package rtc8_gb300 never imports it.
"""
