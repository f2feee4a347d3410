"""GB300-native (sm_103a) rebuild of Spitfire's Griffon chemistry hot path."""
