"""CPU check of the Rust float format used by the tree dump (facts of Rust's `{}` for f64:
shortest round-trip digits, never exponent notation)."""
from treedump import rust_f64


def test_rust_display_of_f64():
    assert rust_f64(1.0) == "1"
    assert rust_f64(0.1) == "0.1"
    assert rust_f64(-0.0) == "-0"
    assert rust_f64(1e-7) == "0.0000001"
    assert rust_f64(1e21) == "1000000000000000000000"
    assert rust_f64(0.30000000000000004) == "0.30000000000000004"
    assert rust_f64(-2.5e-5) == "-0.000025"
    assert rust_f64(123456789.125) == "123456789.125"
    assert rust_f64(float("inf")) == "inf"
