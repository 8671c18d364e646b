"""GB300-native Lindblad `expanded_sparse` solver for CeNTREX-TlF optical Bloch equations."""
