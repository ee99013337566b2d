set output "hist_group1_MOTIF00003.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-19.2687:6.3509]
set yrange [0:195344]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00003.dat" using 1:2 title 'MOTIF00003 (group1)' with boxes
