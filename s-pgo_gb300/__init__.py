"""GB300-native stereo pose-graph / bundle-adjustment LM solver (S-PGO drop-in)."""
