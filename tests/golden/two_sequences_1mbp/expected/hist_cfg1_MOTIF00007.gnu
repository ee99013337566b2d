set output "hist_cfg1_MOTIF00007.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-74.0377:22.6475]
set yrange [0:190289]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00007.dat" using 1:2 title 'MOTIF00007 (cfg1)' with boxes
