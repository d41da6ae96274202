"""GB300-native evaluator for linear ACE models (host side)."""
